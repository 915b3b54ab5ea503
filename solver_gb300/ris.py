"""The dense RIS solver on the GPU (src/lib/solverRis): the reference's entry point
``iter_solver_QS_S_type`` (iter_solver_QS_S_type.jl:1-165) with its operator
``ComputeMatrixVectorRis`` (compute_matrix_vector.jl:1-33) and Householder GMRES
(gmres_custom.jl) running through the C ABI (peec_set_incidence, peec_set_dense and the
solver entry points shared with the voxel path).

The dense Lp and P matrices (``Lp_data``, ``P_data``) are inputs, as they are to the
reference's solver, or are filled on the device from the bodies' vertex coordinates
(``DenseOperator.from_geometry``; ``calcola_Lp`` / ``calcola_P`` return them on the host as
sharedRis/calcola_{Lp,P}.jl do) through peec_ris_fill.

Mapping onto the library's operator: the library forms the first block row as
jw LpI + DZ I + A Phi and the preconditioner with invZ = 1/DZ. With DZ = Z_self +
jw diag(Lp) (the RIS solver's invZ, iter_solver_QS_S_type.jl:103) and LpI the product
with Lp's off-diagonal part (peec_set_dense), that is the RIS operator exactly:
jw Lp I + Z_self I + A Phi. The RIS preconditioner's three LU solves
(compute_matrix_vector.jl:35-57) become one by linearity, as on the voxel path.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import _lib
from .operator import GpuOperator

MU0 = 4 * math.pi * 1e-7
EPS0 = 8.854187816997944e-12


class DenseOperator(GpuOperator):
    """A GPU operator with dense Lp blocks and a dense P over a mesh without voxel
    lattices. Solver entry points (set_frequency, gmres, solve_mixed, port_rhs,
    set_frequency_refactor, ...) are those of GpuOperator; DZ = Z_self + jw diag(Lp)."""

    def __init__(self, incidence_selection, Lp_data, P_data, device=0, geometry=None):
        self.L = _lib.load()
        self._init_args = (incidence_selection, Lp_data, P_data, device)
        self._geometry = geometry
        self._device_dist = False
        self._rows = None
        self._rcc = None
        self._rcc_freq = None
        self._freq_key = None
        self._spec_src = None
        self._stop = None
        self.grid = None
        h = ctypes.c_void_p()
        rc = self.L.peec_ctx_create(ctypes.byref(h), device)
        if rc != 0:
            raise _lib.PeecError(rc, self.L.peec_last_error(None).decode())
        self.h = h
        if not GpuOperator.DEVICE_LOOP:
            self.set_device_loop(False)
        if GpuOperator.LU_COMPONENT_MAX != 512:
            self.set_lu_component_max(GpuOperator.LU_COMPONENT_MAX)
        A = incidence_selection["A"].tocsr()
        Gamma = incidence_selection["Gamma"].tocsc()
        self.m, self.n = A.shape
        self.ns = Gamma.shape[1]
        self.N = self.m + self.ns + self.n
        mx, my, mz = (int(incidence_selection[k]) for k in ("mx", "my", "mz"))
        if mx + my + mz != self.m:
            raise ValueError(f"mx+my+mz={mx + my + mz} must equal the {self.m} rows of A")
        if np.any(np.diff(A.indptr) != 2):
            raise ValueError("A must have two entries per edge row")
        a, b = A.indices[A.indptr[:-1]], A.indices[A.indptr[:-1] + 1]
        va = A.data[A.indptr[:-1]]
        n1 = np.ascontiguousarray(np.where(va < 0, a, b), dtype=np.int64)
        n2 = np.ascontiguousarray(np.where(va < 0, b, a), dtype=np.int64)
        if np.any(np.diff(Gamma.indptr) != 1):
            raise ValueError("Gamma must have one entry per surface column")
        snode = np.ascontiguousarray(Gamma.indices, dtype=np.int64)
        _lib.check(self.h, self.L.peec_set_incidence(self.h, mx, my, mz, _lib.ptr(n1),
                                                     _lib.ptr(n2), self.ns, _lib.ptr(snode),
                                                     self.n))
        if geometry is not None:
            self.fill(*geometry)
            return
        blocks = []
        for key, size in (("Lp_x", mx), ("Lp_y", my), ("Lp_z", mz)):
            M = np.asfortranarray(np.asarray(Lp_data[key], dtype=np.float64))
            if M.shape != (size, size):
                raise ValueError(f"{key} must be {size} x {size}, got {M.shape}")
            blocks.append(M)
        P = np.asfortranarray(np.asarray(P_data["P"], dtype=np.float64))
        if P.shape != (self.ns, self.ns):
            raise ValueError(f"P must be {self.ns} x {self.ns}, got {P.shape}")
        blocks.append(P)
        dP = np.ascontiguousarray(np.diag(P))  # kept referenced while the library reads it
        _lib.check(self.h, self.L.peec_set_pdiag(self.h, _lib.ptr(dP)))
        ptrs = [_lib.ptr(M) if M.size else None for M in blocks]
        _lib.check(self.h, self.L.peec_set_dense(self.h, *ptrs))
        self.diag_Lp = np.concatenate([np.diag(M) for M in blocks[:3]])
        self.diag_P = np.diag(P).copy()

    @classmethod
    def from_geometry(cls, incidence_selection, volumi, superfici, escalings, QS_Rcc_FW=1,
                      device=0):
        """The operator with its Lp blocks and P filled on the device from the bodies'
        vertex coordinates (calcola_Lp.jl / calcola_P.jl through peec_ris_fill); with
        QS_Rcc_FW >= 2 also their centre distances, so that set_rcc_frequency forms the
        retarded blocks without host data."""
        return cls(incidence_selection, None, None, device=device,
                   geometry=(volumi, superfici, escalings, int(QS_Rcc_FW)))

    def fill(self, volumi, superfici, escalings, QS_Rcc_FW=1):
        """(Re)fills the dense blocks on the device from the bodies (peec_ris_fill); with
        QS_Rcc_FW >= 2 also their centre distances."""
        self._geometry = (volumi, superfici, escalings, int(QS_Rcc_FW))
        vol = ris_volumes(volumi, self.m)
        surf = ris_surfaces(superfici, self.ns)
        dist = int(QS_Rcc_FW) >= 2
        bad = ctypes.c_int64(0)
        _lib.check(self.h, self.L.peec_ris_fill(
            self.h, _lib.ptr(vol["coordinate"]), _lib.ptr(vol["S"]),
            _lib.ptr(vol["centri"]) if dist else None, float(escalings["Lp"]),
            _lib.ptr(surf["estremi_celle"]), _lib.ptr(surf["S"]),
            _lib.ptr(surf["centri"]) if dist else None, float(escalings["P"]), int(dist),
            ctypes.byref(bad)))
        self.nonfinite = int(bad.value)
        self._device_dist = dist
        self.diag_Lp = np.concatenate([self.dense_get(b, 2) for b in range(3)])
        self.diag_P = self.dense_get(3, 2)

    def dense_get(self, block, what=0):
        """Block 0..2 (Lp_x, Lp_y, Lp_z) or 3 (P) from the device: what 0 the matrix,
        1 its centre distances, 2 its diagonal."""
        inc = self._init_args[0]
        n = (int(inc["mx"]), int(inc["my"]), int(inc["mz"]), self.ns)[block]
        out = np.zeros(n if what == 2 else (n, n), dtype=np.float64, order="F")
        if n:
            _lib.check(self.h, self.L.peec_dense_get(self.h, int(block), int(what), _lib.ptr(out)))
        return out

    def dense_data(self):
        """(Lp_data, P_data) as calcola_Lp / calcola_P return them: Lp_x, Lp_y, Lp_z (and Rx,
        Ry, Rz when the distances are on the device); P (and R_cc)."""
        Lp = {k: self.dense_get(b) for b, k in enumerate(("Lp_x", "Lp_y", "Lp_z"))}
        P = {"P": self.dense_get(3)}
        if self._device_dist:
            Lp.update({k: self.dense_get(b, 1) for b, k in enumerate(("Rx", "Ry", "Rz"))})
            P["R_cc"] = self.dense_get(3, 1)
        return Lp, P

    def clone(self):
        """A second context with the same mesh and matrices (its own stream and
        workspaces), for concurrent port solves."""
        inc, Lp, P, dev = self._init_args
        c = DenseOperator(inc, Lp, P, device=dev, geometry=self._geometry)
        if getattr(self, "_rcc_dist", None) is not None:
            c.set_rcc(*self._rcc_dist)
        return c

    def set_rcc(self, Lp_data, P_data):
        """The retarded operator (QS_Rcc_FW == 2): the centre distances Lp_data[:Rx],
        [:Ry], [:Rz] and P_data[:R_cc] of the dense blocks; set_rcc_frequency forms the
        blocks times exp(-j beta R) of a frequency on the device. None, None: back to the
        quasi-static blocks."""
        if Lp_data is None and P_data is None:
            _lib.check(self.h, self.L.peec_set_dense_rcc(self.h, None, None, None, None))
            self._rcc_dist = None
            return
        if self._device_dist:
            raise ValueError("the distances of this operator are on the device: "
                             "set_rcc_frequency forms the retarded blocks")
        mats = []
        for key, size in (("Rx", self._init_args[0]["mx"]), ("Ry", self._init_args[0]["my"]),
                          ("Rz", self._init_args[0]["mz"])):
            M = np.asfortranarray(np.asarray(Lp_data[key], dtype=np.float64))
            if M.shape != (int(size), int(size)):
                raise ValueError(f"{key} must be {size} x {size}, got {M.shape}")
            mats.append(M)
        R = np.asfortranarray(np.asarray(P_data["R_cc"], dtype=np.float64))
        if R.shape != (self.ns, self.ns):
            raise ValueError(f"R_cc must be {self.ns} x {self.ns}, got {R.shape}")
        mats.append(R)
        _lib.check(self.h, self.L.peec_set_dense_rcc(self.h, *[_lib.ptr(M) if M.size else None
                                                              for M in mats]))
        self._rcc_dist = (Lp_data, P_data)

    def set_rcc_frequency(self, f_hz):
        """Forms the retarded blocks at frequency f_hz (Hz): beta = 2 pi f sqrt(eps0 mu0)
        (iter_solver_QS_S_type.jl:41-44)."""
        beta = 2 * math.pi * float(f_hz) * math.sqrt(EPS0 * MU0)
        _lib.check(self.h, self.L.peec_set_dense_rcc_frequency(self.h, beta))


def _key(d, name):
    """d[name] for string- or symbol-keyed dicts (the reference's volumi uses symbols,
    superfici strings)."""
    return d[name] if name in d else d[":" + name]


def _rows(a, width, count, name):
    """An array of count rows of width values, row-major: accepts the (count, width)
    matrix or the reference's JSON layout, width lists of count values (what
    hcat(...) turns into the matrix, calcola_P.jl:11-12)."""
    a = np.asarray(a, dtype=np.float64)
    if a.shape == (width, count) and a.shape != (count, width):
        a = a.T
    if a.shape != (count, width):
        raise ValueError(f"{name} must be {count} x {width}, got {a.shape}")
    return np.ascontiguousarray(a)


def ris_volumes(volumi, m):
    """volumi[:coordinate] (m x 24), [:S] (m), [:centri] (m x 3) as contiguous arrays."""
    out = {"coordinate": _rows(_key(volumi, "coordinate"), 24, m, "volumi coordinate"),
           "S": np.ascontiguousarray(np.asarray(_key(volumi, "S"), dtype=np.float64).ravel())}
    if out["S"].size != m:
        raise ValueError(f"volumi S must have {m} entries")
    c = volumi.get("centri", volumi.get(":centri"))
    out["centri"] = _rows(c, 3, m, "volumi centri") if c is not None else np.zeros((m, 3))
    return out


def ris_surfaces(superfici, ns):
    """superfici["estremi_celle"] (ns x 12), ["S"] (ns), ["centri"] (ns x 3)."""
    out = {"estremi_celle": _rows(_key(superfici, "estremi_celle"), 12, ns,
                                  "superfici estremi_celle"),
           "S": np.ascontiguousarray(np.asarray(_key(superfici, "S"), dtype=np.float64).ravel())}
    if out["S"].size != ns:
        raise ValueError(f"superfici S must have {ns} entries")
    c = superfici.get("centri", superfici.get(":centri"))
    out["centri"] = _rows(c, 3, ns, "superfici centri") if c is not None else np.zeros((ns, 3))
    return out


def voxel_bodies(incidence_selection, expansions, grid, cell):
    """The RIS bodies of a voxel mesh, as the RIS solver's inputs describe them: per edge
    the brick of its Lp cell (one voxel length along the edge, between the two voxel
    centres; volumi[:coordinate], [:S] the cross-section, [:centri]) and per surface its
    voxel face (superfici["estremi_celle"], ["S"] the area, ["centri"]). cell = (sx, sy,
    sz); lattice origin at 0."""
    from .operator import _edge_cells, _surf_cells, row_dims
    mx, my, mz = (int(incidence_selection[k]) for k in ("mx", "my", "mz"))
    ns = incidence_selection["Gamma"].shape[1]
    Nx, Ny, Nz = grid[:3]
    cell = np.asarray(cell, dtype=np.float64)
    dims = row_dims(Nx, Ny, Nz)

    def ijk(ids, d):
        ids = np.asarray(ids, dtype=np.int64)
        return np.stack([ids % d[0], (ids // d[0]) % d[1], ids // (d[0] * d[1])],
                        axis=1).astype(np.float64)

    def corners(lo, hi):
        # vertex k at (x, y, z) bits (k & 1, k >> 1 & 1, k >> 2): the reference's order
        out = np.empty((lo.shape[0], 8, 3))
        for k in range(8):
            for a in range(3):
                out[:, k, a] = hi[:, a] if (k >> a) & 1 else lo[:, a]
        return out

    ec = _edge_cells(expansions, mx, my, mz)
    los, S = [], []
    for d, (key, sl) in enumerate((("Lpx", slice(0, mx)), ("Lpy", slice(mx, mx + my)),
                                   ("Lpz", slice(mx + my, mx + my + mz)))):
        lo = ijk(ec[sl], dims[key])
        lo[:, d] += 0.5
        los.append(lo)
        t = [q for q in range(3) if q != d]
        S.append(np.full(lo.shape[0], cell[t[0]] * cell[t[1]]))
    lo = np.concatenate(los) * cell
    hi = lo + cell
    volumi = {"coordinate": corners(lo, hi).reshape(-1, 24), "S": np.concatenate(S),
              "centri": 0.5 * (lo + hi)}
    fam, scell = _surf_cells(expansions, ns)
    lo = np.zeros((ns, 3))
    nrm = np.array([1, 0, 2])[fam]
    for f, key in enumerate(("p12_se", "p34_se", "p56_se")):
        sel = fam == f
        lo[sel] = ijk(scell[sel], dims[key])
    lo = lo * cell
    ext = np.tile(cell, (ns, 1))
    ext[np.arange(ns), nrm] = 0.0
    hi = lo + ext
    area = np.prod(np.where(ext > 0, ext, 1.0), axis=1)
    ends = np.zeros((ns, 12))
    ends[:, 0:3] = lo
    ends[:, 9:12] = hi
    ends[:, 3:6] = np.where(np.arange(3) == (nrm[:, None] + 1) % 3, hi, lo)
    ends[:, 6:9] = np.where(np.arange(3) == (nrm[:, None] + 2) % 3, hi, lo)
    superfici = {"estremi_celle": ends, "S": area, "centri": 0.5 * (lo + hi)}
    return volumi, superfici


def _sizes_only(mx, my, mz, ns):
    """An incidence_selection that carries only the block sizes (every edge on one node,
    every surface on it), for a context that only fills and returns dense blocks."""
    inc = {"mx": mx, "my": my, "mz": mz,
           "A": sp.csr_matrix((np.tile([-1.0, 1.0], mx + my + mz),
                               np.zeros(2 * (mx + my + mz), dtype=np.int64),
                               np.arange(0, 2 * (mx + my + mz) + 1, 2)), shape=(mx + my + mz, 1)),
           "Gamma": sp.csc_matrix((np.ones(ns), np.zeros(ns, dtype=np.int64), np.arange(ns + 1)),
                                  shape=(1, ns))}
    return inc


def calcola_Lp(volumi, incidence_selection, escalings, QS_Rcc_FW, device=0):
    """calcola_Lp (sharedRis/calcola_Lp.jl:1-97) on the GPU: the dense Lp_x, Lp_y, Lp_z
    (and Rx, Ry, Rz when QS_Rcc_FW >= 2), returned on the host, with "nonfinite" the
    count of non-finite entries. For QS_Rcc_FW < 2 the reference's function reads its
    unassigned Rx at the return and raises; here the distances are left out."""
    mx, my, mz = (int(incidence_selection[k]) for k in ("mx", "my", "mz"))
    inc = _sizes_only(mx, my, mz, 0)
    op = DenseOperator(inc, None, None, device=device,
                       geometry=(volumi, {"estremi_celle": np.zeros((0, 12)), "S": np.zeros(0)},
                                 escalings, int(QS_Rcc_FW)))
    try:
        Lp, _ = op.dense_data()
        Lp["nonfinite"] = op.nonfinite
        return Lp
    finally:
        op.close()


def calcola_P(superfici, escalings, QS_Rcc_FW, device=0):
    """calcola_P (sharedRis/calcola_P.jl:1-47) on the GPU: the dense P (and R_cc when
    QS_Rcc_FW >= 2), returned on the host, with "nonfinite" the count of non-finite
    entries. For QS_Rcc_FW < 2 the reference returns R_cc = nothing into a matrix-typed
    Dict and raises; here R_cc is left out."""
    ns = len(np.asarray(_key(superfici, "S")).ravel())
    inc = _sizes_only(0, 0, 0, ns)
    op = DenseOperator(inc, None, None, device=device,
                       geometry=({"coordinate": np.zeros((0, 24)), "S": np.zeros(0)}, superfici,
                                 escalings, int(QS_Rcc_FW)))
    try:
        _, P = op.dense_data()
        P["nonfinite"] = op.nonfinite
        return P
    finally:
        op.close()


def find_nodes_ports_or_le(port_objects, lumped_elements_objects, nodi_coord, escal):
    """find_nodes_ports_or_le (sharedRis/find_nodes_ports_or_le.jl:1-103): each port's and
    lumped element's terminal positions, every coordinate rounded to 5 decimals then scaled
    by escal, mapped to the first node at the smallest Euclidean distance (nodes_find_rev
    with distfcm, :105-119). Returns (ports, lumped_elements) in the form the RIS loop
    takes, node indices 0-based."""
    nodes = np.asarray(nodi_coord, dtype=np.float64)
    if nodes.ndim == 2 and nodes.shape[0] == 3 and nodes.shape[1] != 3:
        nodes = nodes.T  # the JSON layout: three lists of node coordinates
    nodes = nodes.reshape(-1, 3)

    def pos(p):
        return np.array([np.rint(float(p[i]) * 1e5) / 1e5 * escal for i in range(3)])

    def nearest(q):
        d = np.sqrt(((nodes - q) ** 2).sum(axis=1))
        return int(np.flatnonzero(d == d.min())[0])

    def terminals(objs):
        return np.array([[nearest(pos(o["inputElement"])), nearest(pos(o["outputElement"]))]
                         for o in objs], dtype=np.int64).reshape(-1, 2)

    ports = {"port_start": [pos(o["inputElement"]) for o in port_objects],
             "port_end": [pos(o["outputElement"]) for o in port_objects],
             "port_nodes": terminals(port_objects)}
    les = list(lumped_elements_objects or [])
    rlc = lambda o, k: float(o.get("rlcParams", {}).get(k, 0.0))
    lumped = {"le_start": [pos(o["inputElement"]) for o in les],
              "le_end": [pos(o["outputElement"]) for o in les],
              "le_nodes": terminals(les), "type": [o["type"] for o in les],
              "R": [rlc(o, "resistance") for o in les], "L": [rlc(o, "inductance") for o in les],
              "C": [rlc(o, "capacitance") for o in les]}
    return ports, lumped


def do_solving_ris(incidence_selection, volumi, superfici, nodi_coord, escalings, solverInput,
                   solverAlgoParams, solverType, mode="fp64", device=0, lu="host"):
    """doSolvingRis (solverRis/do_solving_ris.jl:1-78) without its service parts (S3, AMQP,
    stop flags): ports and lumped elements mapped to nodes, the dense Lp blocks and P filled
    on the GPU, and the frequency x port loop (GMRES settings from solverAlgoParams; 1e-8
    below 100 kHz; QS_Rcc_FW = solverType; surface impedance on). Returns the loop's dict
    (S, Z, Y, f)."""
    from .mesher import get_escal_from
    escal = get_escal_from(solverInput.get("unit", "m"))
    R = float(solverInput.get("ports_scattering_value", 50.0))
    freq = np.asarray(solverInput["frequencies"], dtype=np.float64).ravel()
    ports, le = find_nodes_ports_or_le(solverInput["ports"], solverInput.get("lumped_elements", []),
                                       nodi_coord, escal)
    tol = float(solverAlgoParams["convergenceThreshold"]) * np.ones(freq.size)
    tol[freq < 1e5] = 1e-8
    gs = {"Inner_Iter": int(solverAlgoParams["innerIteration"]),
          "Outer_Iter": int(solverAlgoParams["outerIteration"]), "tol": tol}
    op = DenseOperator.from_geometry(incidence_selection, volumi, superfici, escalings,
                                     int(solverType), device=device)
    try:
        return iter_solver_QS_S_type(freq, escalings, incidence_selection, None, None, ports, le,
                                     gs, volumi, True, int(solverType), R, mode=mode, op=op, lu=lu)
    finally:
        op.close()


def lumped_admittance_S(typ, R, L, C, w):
    """get_lumped_elements_admittance_S (build_Yle_S.jl:70-151): the element's network,
    then while the value is not finite or below 1e-16 in magnitude the next network of the
    cascade (IEEE divisions by zero, as in Julia). The RIS cascade of type 2 differs from
    the voxel path's in its fifth network: 1/(1/(jwC)) + jwC."""
    R, L, C = np.float64(R), np.float64(L), np.float64(C)
    jw = np.complex128(1j * w)
    bad = lambda v: np.isnan(v) or np.isinf(v) or abs(v) < 1e-16
    with np.errstate(all="ignore"):
        if typ == 1:
            z = R + jw * L + 1 / (jw * C)
            if bad(z):
                z = R + jw * L
            y = 1 / z
        else:
            nets = {
                2: (lambda: 1 / (R + jw * L) + jw * C, lambda: 1 / R + jw * C,
                    lambda: 1 / (R + jw * L), lambda: 1 / R,
                    lambda: 1 / (1 / (jw * C)) + jw * C, lambda: jw * C),
                3: (lambda: 1 / (R + 1 / (jw * C)) + 1 / (jw * L), lambda: 1 / (R + 1 / (jw * C)),
                    lambda: 1 / R + 1 / (jw * L), lambda: 1 / R,
                    lambda: 1 / (1 / (jw * C)) + 1 / (jw * L), lambda: 1 / (jw * L),
                    lambda: 1 / (1 / (jw * C))),
                4: (lambda: 1 / R + jw * C + 1 / (jw * L), lambda: 1 / R + jw * C,
                    lambda: jw * C + 1 / (jw * L), lambda: jw * C),
                5: (lambda: 1 / R + 1 / (jw * L + 1 / (jw * C)), lambda: 1 / R + 1 / (1 / (jw * C)),
                    lambda: 1 / R + 1 / (jw * L), lambda: 1 / R,
                    lambda: 1 / (jw * L + 1 / (jw * C)), lambda: 1 / (jw * L),
                    lambda: 1 / (1 / (jw * C))),
            }.get(int(typ), (lambda: np.complex128(0.0),))
            y = nets[0]()
            for f in nets[1:]:
                if not bad(y):
                    break
                y = f()
        if np.isnan(y) or np.isinf(y):
            y = 0.0
    return complex(y)


def build_yle_s(lumped_elements, grounding_nodes, ports, escalings, n, w, val_chiusura):
    """Sparse n x n admittance of the lumped elements, the port closures (1/R between each
    port's nodes) and the grounding nodes (1e-12), summed per entry and scaled by
    escalings["Yle"] (build_Yle_S.jl:1-68). Complex element admittances stay complex (the
    reference sums into a Float64 dictionary, which holds real ones only)."""
    acc = {}

    def add(r, c, v):
        acc[(r, c)] = acc.get((r, c), 0.0) + v

    le = lumped_elements or {}
    for k in range(len(le.get("le_nodes", []))):
        a, b = int(le["le_nodes"][k][0]), int(le["le_nodes"][k][1])
        y = lumped_admittance_S(le["type"][k], le["R"][k], le["L"][k], le["C"][k], w)
        add(a, a, y)
        add(b, b, y)
        add(a, b, -y)
        add(b, a, -y)
    for k in range(len(ports["port_nodes"])):
        a, b = int(ports["port_nodes"][k][0]), int(ports["port_nodes"][k][1])
        y = 1.0 / val_chiusura
        add(a, a, y)
        add(b, b, y)
        add(a, b, -y)
        add(b, a, -y)
    for g in grounding_nodes:
        add(int(g), int(g), 1.0 / 1e12)
    if not acc:
        return sp.csr_matrix((n, n), dtype=np.complex128)
    rc = np.array(list(acc.keys()), dtype=np.int64)
    v = np.array(list(acc.values()), dtype=np.complex128) * escalings["Yle"]
    return sp.csr_matrix((v, (rc[:, 0], rc[:, 1])), shape=(n, n))


def z_self(volumi, w, use_Zs_in):
    """Self impedance per edge (iter_solver_QS_S_type.jl:82-101): R, or with use_Zs_in the
    surface impedance Re(sqrt(jw) Zs_part) where it is not below R; plus 1/(jw Cd) on the
    dielectric volumes."""
    R = np.asarray(_key(volumi, "R"), dtype=np.float64).ravel()
    diel = np.asarray(volumi.get("indici_dielettrici", volumi.get(":indici_dielettrici", [])),
                      dtype=np.int64).ravel()
    invCd = np.zeros(len(_key(volumi, "Cd")) if diel.size else R.size, dtype=np.complex128)
    if diel.size:
        Cd = np.asarray(_key(volumi, "Cd"), dtype=np.float64).ravel()
        invCd[diel] = 1.0 / (1j * w * Cd[diel])
    if use_Zs_in:
        Zs = (np.sqrt(1j * w) * np.asarray(_key(volumi, "Zs_part"), dtype=np.complex128).ravel()).real
        Z = np.where(R > Zs, R, Zs).astype(np.complex128)
        return Z + invCd
    return R + invCd


class RisState:
    """One frequency's host state: Z_self, DZ = Z_self + jw diag(Lp), Yle and the LU of
    SS = Yle + A' diag(1/DZ) A + jw Gamma diag(1/P) Gamma' (iter_solver_QS_S_type.jl:82-115)."""

    def __init__(self, w, escalings, incidence_selection, diag_Lp, diag_P, ports,
                 lumped_elements, volumi, use_Zs_in, val_chiusura, factor=True):
        A = incidence_selection["A"]
        Gamma = incidence_selection["Gamma"]
        n = A.shape[1]
        self.w = w
        self.Yle = build_yle_s(lumped_elements, [], ports, escalings, n, w / escalings["freq"],
                               val_chiusura)
        self.Z_self = z_self(volumi, w, use_Zs_in)
        self.DZ = self.Z_self + 1j * w * np.asarray(diag_Lp, dtype=np.float64)
        self.lu = None
        if factor:
            invZ = sp.diags(1.0 / self.DZ)
            invP = sp.diags(1.0 / np.asarray(diag_P, dtype=np.float64))
            SS = (self.Yle + A.T @ (invZ @ A) + 1j * w * ((Gamma @ invP) @ Gamma.T)).tocsc()
            self.lu = spla.splu(SS, permc_spec="MMD_AT_PLUS_A", options={"Equil": False})


def iter_solver_QS_S_type(freq, escalings, incidence_selection, P_data, Lp_data, ports,
                          lumped_elements, GMRES_settings, volumi, use_Zs_in, QS_Rcc_FW,
                          ports_scatter_value, mode="fp64", op=None, device=0, lu="host"):
    """The RIS solver's frequency x port loop on the GPU (iter_solver_QS_S_type.jl:1-165):
    per frequency the state, per port the right-hand side M^-1 [0; 0; is], GMRES warm
    started from that port's previous solution, and the S entries
    S(c1,c2) = (2 (V(n3) - V(n4)) - R delta) / R. mode "fp64": the reference's FP64 GMRES;
    "mixed": FP32 dense products with float-float / FP64 refinement. lu="device": SS is
    factorised on the GPU after the first frequency, in that frequency's pattern.
    Returns the reference's dict (S, Z, Y, f) plus the per-solve records (info)."""
    if int(QS_Rcc_FW) not in (1, 2):
        raise NotImplementedError("QS_Rcc_FW must be 1 (quasi-static) or 2 (retarded)")
    rcc = int(QS_Rcc_FW) == 2
    if mode not in ("fp64", "mixed"):
        raise ValueError("mode must be 'fp64' or 'mixed'")
    freq = np.asarray(freq, dtype=np.float64).ravel() * escalings["freq"]
    A = incidence_selection["A"]
    m, n = A.shape
    ns = incidence_selection["Gamma"].shape[1]
    pn = np.asarray(ports["port_nodes"], dtype=np.int64).reshape(-1, 2)
    npt = pn.shape[0]
    R = float(ports_scatter_value)
    own = op is None
    if own:
        op = DenseOperator(incidence_selection, Lp_data, P_data, device=device)
    if rcc and not op._device_dist:
        op.set_rcc(Lp_data, P_data)
    diag_P = op.diag_P
    S = np.zeros((npt, npt, freq.size), dtype=np.complex128)
    Vrest = np.zeros((m + ns + n, npt), dtype=np.complex128)
    info = []
    tol = np.broadcast_to(np.asarray(GMRES_settings["tol"], dtype=np.float64), freq.shape)
    maxit = int(GMRES_settings["Inner_Iter"])
    try:
        for k, f in enumerate(freq):
            w = 2 * math.pi * f
            dev_lu = lu == "device" and k > 0
            if rcc:
                # the retarded blocks of this frequency (their diagonals are the quasi-static
                # ones: the distances are zero there)
                op.set_rcc_frequency(f / escalings["freq"])
            st = RisState(w, escalings, incidence_selection, op.diag_Lp, diag_P, ports,
                          lumped_elements, volumi, use_Zs_in, R, factor=not dev_lu)
            if dev_lu:
                op.set_frequency_refactor(w, st.DZ, st.Yle)
            else:
                op.set_frequency(w, st.DZ, st.Yle, st.lu)
                if lu == "device":
                    op.enable_refactor(st.Yle)
            for c1 in range(npt):
                n1, n2 = pn[c1]
                tn = op.port_rhs(n1, n2, escalings["Is"])
                x0 = Vrest[:, c1]
                if mode == "fp64":
                    V, flag, relres, it, rv = op.gmres(tn, x0, float(tol[k]), maxit)
                    rec = dict(freq=k, port=c1, flag=flag, relres=relres, iter=list(it),
                               niter=len(rv) - 1)
                else:
                    V, flag, relres, outer, inner = op.solve_mixed(tn, x0, float(tol[k]),
                                                                   inner_maxit=maxit)
                    rec = dict(freq=k, port=c1, flag=flag, relres=relres, outer=outer,
                               niter=inner)
                info.append(rec)
                Vrest[:, c1] = V
                for c2 in range(c1, npt):
                    n3, n4 = pn[c2]
                    d = 2 * (V[m + ns + n3] - V[m + ns + n4])
                    S[c1, c2, k] = (d - R) / R if c1 == c2 else d / R
                    S[c2, c1, k] = S[c1, c2, k]
    finally:
        if own:
            op.close()
        elif rcc:
            op.set_rcc(None, None)  # back to the quasi-static blocks for later users
            # (with the distances on the device, set_rcc_frequency returns to the retarded ones)
    Id = np.eye(npt)
    Z = np.stack([R * np.linalg.solve(Id - S[:, :, k], Id + S[:, :, k]) for k in range(freq.size)],
                 axis=2) if freq.size else S.copy()
    Y = np.stack([R * np.linalg.solve(Id + S[:, :, k], Id - S[:, :, k]) for k in range(freq.size)],
                 axis=2) if freq.size else S.copy()
    return {"S": S, "Z": Z, "Y": Y, "f": freq / escalings["freq"], "info": info, "Vrest": Vrest}
