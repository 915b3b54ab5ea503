"""Dense CPU solves of a one-port geometry for the gradient tests: the oracle's FFT
operator (ComputeMatrixVectorFTT restated in oracle/peec_oracle.py) assembled column by
column into a dense matrix and solved by LU, at per-voxel conductivities. Test
infrastructure: only the tests import it."""
import numpy as np
import scipy.sparse as sp

from oracle import peec_oracle as O
from solver_gb300 import frequency as fq, gradient as G, mesher


class DensePort:
    def __init__(self, req):
        out, self.freqs, _settings, self.z0, grid = mesher.parse_request(req)
        (self.esc, self.inc, self.cc, self.diag, self.exp, self.ports, self.le, _li,
         self.Zs) = out
        rows = O.fill_rows(self.cc, self.esc, *grid)
        self.FP, self.FL = O.spectra_from_rows(rows, *grid)
        self.m, self.n = self.inc["A"].shape
        self.ns = self.inc["Gamma"].shape[1]
        self.v1, self.v2 = G.edge_voxels(self.inc, self.exp)
        self.nvox = int(np.max(self.exp["vox_map"]))
        mats = np.asarray(self.Zs["materials"], dtype=np.int64)
        self.sigma_edge = G.edge_sigma(self.Zs, [5.8e7] * int(mats.max()))
        self.sigma_ref = np.zeros(self.nvox)
        c = self.sigma_edge > 0
        self.sigma_ref[self.v1[c]] = self.sigma_edge[c]
        self.sigma_ref[self.v2[c]] = self.sigma_edge[c]

    def solve(self, k, sigma_voxel=None):
        """|Z|, d|Z|/d sigma (reciprocity) and Z from a dense LU solve at frequency k."""
        sv = self.sigma_ref if sigma_voxel is None else sigma_voxel
        w = 2 * np.pi * self.freqs[k] * self.esc["freq"]
        DZ, d1, d2 = G.dz_edges(w, self.esc, self.diag, self.Zs, sv, self.v1, self.v2,
                               self.sigma_edge)
        st = fq.FrequencyState(w, self.esc, self.inc, self.diag, self.Zs, self.le,
                               self.ports, self.z0, DZ=DZ)
        fo = O.frequency_setup(w, self.esc, self.inc, self.diag, self.Zs, self.le,
                               self.ports, self.z0)
        fo["DZ"], fo["invZ"], fo["F"] = st.DZ, sp.diags(1 / st.DZ), st.lu.solve
        N = self.m + self.ns + self.n
        A = O.dense_operator(lambda x: O.ComputeMatrixVectorFTT(
            x, w, self.inc, self.FP, self.FL, fo["DZ"], fo["Yle"], self.exp, fo["invZ"],
            fo["invP"], fo["F"]), N)
        n1, n2 = self.ports["port_nodes"][0]
        i_s = np.zeros(self.n)
        i_s[n1], i_s[n2] = self.esc["Is"], -self.esc["Is"]
        tn = O.precond_3_3_Kt_fft(fo["F"], fo["invZ"], fo["invP"], self.inc["A"],
                                  self.inc["Gamma"], self.m, self.ns, i_s)
        V = np.linalg.solve(A, tn)
        return G.port_impedance_and_gradient(V, self.m, self.ns, (n1, n2), self.z0,
                                             self.esc["Is"], d1, d2, self.v1, self.v2,
                                             self.nvox)

    def finite_difference(self, k, voxels, h_rel):
        out = []
        for v in voxels:
            h = h_rel * self.sigma_ref[v]
            vals = []
            for sgn in (1.0, -1.0):
                sv = self.sigma_ref.copy()
                sv[v] += sgn * h
                vals.append(self.solve(k, sv)[0])
            out.append((vals[0] - vals[1]) / (2 * h))
        return np.asarray(out)


def bar_request(freqs, shape=(12, 12, 6)):
    """A copper bar (shape[0] x 2 x 2 voxels) joining the port terminals, with
    Bernoulli(0.2) copper clutter around it (seed 7), on a grid of 5e-5 m voxels."""
    from solver_gb300 import configs
    rng = np.random.default_rng(7)
    cu = configs.drop_isolated(rng.random(shape) < 0.2)
    y, z = shape[1] // 2 - 1, shape[2] // 2 - 1
    cu[:, y:y + 2, z:z + 2] = True
    return configs.make_request({"copper": cu}, [dict(configs.COPPER)], (5e-5,) * 3,
                                [((0, y, z), (shape[0] - 1, y, z))], freqs, 1e-10)
