"""GPU operator: one geometry's circulant Lp/P operator and preconditioner on a GB300.

Wraps a ``peec_ctx`` (include/peec_gb300.h). Everything that touches vectors of
length N = m + ns + n runs in the CUDA library; this class only converts the
reference's host data structures into the C ABI's flat arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.sparse as sp

from . import _lib
from .frequency import export_lu

ROW_KEYS = ("Lpx", "Lpy", "Lpz", "p12_se", "p34_se", "p56_se", "p1234", "p1256", "p3456")


def row_dims(Nx, Ny, Nz):
    return {"Lpx": (Nx - 1, Ny, Nz), "Lpy": (Nx, Ny - 1, Nz), "Lpz": (Nx, Ny, Nz - 1),
            "p12_se": (Nx, Ny + 1, Nz), "p34_se": (Nx + 1, Ny, Nz), "p56_se": (Nx, Ny, Nz + 1),
            "p1234": (2 * Nx + 1, 2 * Ny + 1, Nz), "p1256": (Nx, 2 * Ny + 1, 2 * Nz + 1),
            "p3456": (2 * Nx + 1, Ny, 2 * Nz + 1)}


def _edge_cells(expansions, mx, my, mz):
    """Lattice cell of every edge from mat_map_Lp[c][0] (one 1 per column)."""
    if "edge_cell" in expansions:
        return np.ascontiguousarray(expansions["edge_cell"], dtype=np.int64)
    out = []
    for c, mc in enumerate((mx, my, mz)):
        M = expansions["mat_map_Lp"][c][0].tocsc()
        if M.shape[1] != mc or np.any(np.diff(M.indptr) != 1):
            raise ValueError("mat_map_Lp must hold exactly one 1 per edge column")
        out.append(M.indices.astype(np.int64))
    return np.concatenate(out)


def _surf_cells(expansions, ns):
    if "surf_cell" in expansions and "surf_fam" in expansions:
        return (np.ascontiguousarray(expansions["surf_fam"], dtype=np.int32),
                np.ascontiguousarray(expansions["surf_cell"], dtype=np.int64))
    fam = np.full(ns, -1, dtype=np.int32)
    cell = np.full(ns, -1, dtype=np.int64)
    for f in range(3):
        M = expansions["exp_P"][f][f].tocsc()
        cols = np.nonzero(np.diff(M.indptr))[0]
        if np.any(np.diff(M.indptr)[cols] != 1):
            raise ValueError("exp_P[f][f] must hold at most one 1 per surface column")
        fam[cols] = f
        cell[cols] = M.indices[M.indptr[cols]]
    if np.any(fam < 0):
        raise ValueError("every surface must belong to one face family")
    return fam, cell


class GpuOperator:
    """Device-resident PEEC operator for one geometry."""

    # settings every new context starts with (process-wide; the library's defaults): the
    # device-resident GMRES loop, and the largest LU component solved per warp group
    DEVICE_LOOP = True
    LU_COMPONENT_MAX = 512

    def __init__(self, incidence_selection, expansions, diagP, grid=None, device=0):
        self.L = _lib.load()
        self._init_args = (incidence_selection, expansions, diagP, grid, device)
        self._rows = None
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
        if grid is None:
            grid = expansions["grid"]
        self.grid = tuple(int(v) for v in grid)
        ecell = _edge_cells(expansions, mx, my, mz)
        if mx + my + mz != self.m or ecell.size != self.m:
            raise ValueError(f"edge counts mx+my+mz={mx + my + mz} and {ecell.size} edge cells "
                             f"must both equal the {self.m} rows of A")
        # A rows hold -1 at n1 and +1 at n2
        n1 = np.empty(self.m, dtype=np.int64)
        n2 = np.empty(self.m, dtype=np.int64)
        for e0, e1 in ((0, self.m),):
            ind, dat, ptr = A.indices, A.data, A.indptr
            if np.any(np.diff(ptr) != 2):
                raise ValueError("A must have two entries per edge row")
            a = ind[ptr[:-1]]
            b = ind[ptr[:-1] + 1]
            va = dat[ptr[:-1]]
            n1[:] = np.where(va < 0, a, b)
            n2[:] = np.where(va < 0, b, a)
        if np.any(np.diff(Gamma.indptr) != 1):
            raise ValueError("Gamma must have one entry per surface column")
        snode = Gamma.indices.astype(np.int64)
        fam, scell = _surf_cells(expansions, self.ns)
        if fam.size != self.ns or scell.size != self.ns:
            raise ValueError("surf_fam and surf_cell need one entry per surface")
        Nx, Ny, Nz = self.grid
        _lib.check(self.h, self.L.peec_set_topology(
            self.h, Nx, Ny, Nz, mx, my, mz, _lib.ptr(ecell), _lib.ptr(n1), _lib.ptr(n2), self.ns,
            _lib.ptr(fam), _lib.ptr(scell), _lib.ptr(snode), self.n))
        dp = np.ascontiguousarray(np.asarray(diagP, dtype=np.float64).ravel())
        if dp.size != self.ns:
            raise ValueError(f"diagP has {dp.size} entries, expected {self.ns}")
        _lib.check(self.h, self.L.peec_set_pdiag(self.h, _lib.ptr(dp)))
        self._freq_key = None
        self._spec_src = None  # the host spectra the device rows were recovered from
        self._stop = None
        self._rcc = None  # (rows, origin, (sx, sy, sz)) of the retarded operator, for clone()
        self._rcc_freq = None

    def close(self):
        if getattr(self, "h", None):
            self.L.peec_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- circulant blocks ----------------------------------------------------------
    def set_rows(self, rows: dict):
        """Upload the nine generating rows (escaled, reference lattices, x fastest)."""
        dims = row_dims(*self.grid)
        keep = []
        arr = (ctypes.c_void_p * 9)()
        for i, k in enumerate(ROW_KEYS):
            n = int(np.prod(dims[k]))
            if n == 0 or k not in rows:
                arr[i] = None
                continue
            r = np.ascontiguousarray(np.asarray(rows[k], dtype=np.float64).ravel())
            if r.size != n:
                raise ValueError(f"row {k} has {r.size} entries, expected {n}")
            keep.append(r)
            arr[i] = r.ctypes.data
        self._spec_src = None
        self._rcc_freq = None
        _lib.check(self.h, self.L.peec_set_rows(self.h, arr))
        self._rows = {k: v for k, v in rows.items()}

    def fill(self, origin, sx, sy, sz, escal_Lp, escal_P, return_rows=False):
        """GPU fill of the nine rows and their spectra."""
        dims = row_dims(*self.grid)
        o = np.ascontiguousarray(np.asarray(origin, dtype=np.float64))
        outs = {}
        arr = (ctypes.c_void_p * 9)()
        for i, k in enumerate(ROW_KEYS):
            n = int(np.prod(dims[k]))
            if n > 0:
                outs[k] = np.empty(n)
                arr[i] = outs[k].ctypes.data
            else:
                arr[i] = None
        self._spec_src = None
        self._rcc_freq = None
        _lib.check(self.h, self.L.peec_fill(self.h, _lib.ptr(o), sx, sy, sz, escal_Lp, escal_P,
                                            arr))
        self._rows = outs  # kept for clone()
        return outs if return_rows else None

    # -- retarded (Rcc) operator ------------------------------------------------------
    def _row_buffers(self, rows=None):
        dims = row_dims(*self.grid)
        arr = (ctypes.c_void_p * 9)()
        keep = {}
        for i, k in enumerate(ROW_KEYS):
            n = int(np.prod(dims[k]))
            if n == 0:
                arr[i] = None
                continue
            if rows is None:
                keep[k] = np.empty(n)
            else:
                if k not in rows:
                    raise ValueError(f"missing Rcc row {k}")
                keep[k] = np.ascontiguousarray(np.asarray(rows[k], dtype=np.float64).ravel())
                if keep[k].size != n:
                    raise ValueError(f"row {k} has {keep[k].size} entries, expected {n}")
            arr[i] = keep[k].ctypes.data
        return arr, keep

    def fill_rcc(self, origin, sx, sy, sz, escal_Lp, escal_P):
        """GPU fill of the quasi-static parts of the nine Rcc rows (compute_rows_Rcc_Lp,
        compute_rows_Rcc_P; escaled, Lp self entries zero). Returns the rows."""
        o = np.ascontiguousarray(np.asarray(origin, dtype=np.float64))
        arr, outs = self._row_buffers()
        _lib.check(self.h, self.L.peec_fill_rcc(self.h, _lib.ptr(o), sx, sy, sz, escal_Lp,
                                                escal_P, arr))
        self._rcc = (outs, o.copy(), (float(sx), float(sy), float(sz)))
        self._rcc_freq = None
        return outs

    def set_rows_rcc(self, rows, origin, sx, sy, sz):
        """Uploads the quasi-static parts of the nine Rcc rows (escaled) and the mesh
        geometry their centre distances come from."""
        o = np.ascontiguousarray(np.asarray(origin, dtype=np.float64))
        arr, keep = self._row_buffers(rows)
        _lib.check(self.h, self.L.peec_set_rows_rcc(self.h, arr, _lib.ptr(o), float(sx),
                                                    float(sy), float(sz)))
        self._rcc = (keep, o.copy(), (float(sx), float(sy), float(sz)))
        self._rcc_freq = None

    def set_rcc_frequency(self, freq_hz):
        """The Rcc spectra at freq_hz (Hz); later operator applications use them."""
        if self._rcc_freq is not None and self._rcc_freq == float(freq_hz):
            return
        self._rcc_freq = None
        _lib.check(self.h, self.L.peec_set_rcc_frequency(self.h, float(freq_hz)))
        self._rcc_freq = float(freq_hz)

    def clone(self):
        """A second context on the same device with the same topology and circulant
        rows: its own CUDA stream and workspaces, so several port solves of one
        frequency run concurrently (one context per port, each driven from its own
        host thread). The frequency state (and the Rcc frequency) is set per context."""
        if self._rows is None and self._rcc is None:
            raise RuntimeError("clone() needs the generating rows: call fill, set_rows, "
                               "fill_rcc or set_rows_rcc first")
        inc, exp, dP, grid, dev = self._init_args
        c = GpuOperator(inc, exp, dP, grid=grid, device=dev)
        if self._rows is not None:
            c.set_rows(self._rows)
        if self._rcc is not None:
            rows, o, (sx, sy, sz) = self._rcc
            c.set_rows_rcc(rows, o, sx, sy, sz)
        # the same FP32 z-pass forms as this context (the tuner's timings can differ by a
        # few percent between contexts), so that every lane computes the same numbers
        t = self.zpass_tuning()
        c.set_zpass_forms(t["face"], t["edge"], t["edge_plan"])
        return c

    # -- frequency ------------------------------------------------------------------
    @staticmethod
    def _same_key(a, b):
        """Keys are tuples of scalars and host objects; objects match by identity. A key
        keeps its objects alive, so an identity cannot be reused while it is cached."""
        if a is None or b is None or len(a) != len(b):
            return False
        return all(x is y or (isinstance(x, (int, float, str)) and type(x) is type(y) and x == y)
                   for x, y in zip(a, b))

    def set_frequency(self, w, DZ, Yle, lu, key=None):
        """Uploads one frequency's state. With a key (a tuple of scalars and the host
        objects the state came from), a repeated call with the same key is skipped."""
        if key is not None and self._same_key(key, self._freq_key):
            return
        DZ = np.ascontiguousarray(np.asarray(DZ, dtype=np.complex128).ravel())
        if DZ.size != self.m:
            raise ValueError(f"DZ has {DZ.size} entries, expected {self.m}")
        if tuple(Yle.shape) != (self.n, self.n):
            raise ValueError(f"Yle must be {self.n} x {self.n}")
        Y = sp.coo_matrix(Yle)
        yr = Y.row.astype(np.int64)
        yc = Y.col.astype(np.int64)
        yv = np.ascontiguousarray(Y.data.astype(np.complex128))
        self._freq_key = None  # a failed upload leaves no usable state behind
        (Lp, Lc, Lv), (Up, Uc, Uv), pr, pc = export_lu(lu)
        for ptr, col, val in ((Lp, Lc, Lv), (Up, Uc, Uv)):
            if ptr.size != self.n + 1 or ptr[-1] != col.size or val.size != 2 * col.size:
                raise ValueError(f"LU factors must be {self.n} x {self.n} CSR")
        if pr.size != self.n or pc.size != self.n:
            raise ValueError(f"LU permutations need {self.n} entries")
        _lib.check(self.h, self.L.peec_set_frequency(
            self.h, float(w), _lib.ptr(DZ.view(np.float64)), int(yr.size), _lib.ptr(yr),
            _lib.ptr(yc), _lib.ptr(yv.view(np.float64)), _lib.ptr(Lp), _lib.ptr(Lc), _lib.ptr(Lv),
            _lib.ptr(Up), _lib.ptr(Uc), _lib.ptr(Uv), _lib.ptr(pr), _lib.ptr(pc), None))
        self._freq_key = key

    @staticmethod
    def _yle_coo(Yle):
        Y = sp.coo_matrix(Yle)
        return (Y.row.astype(np.int64), Y.col.astype(np.int64),
                np.ascontiguousarray(Y.data.astype(np.complex128)))

    def enable_refactor(self, Yle):
        """Later frequencies may factorise SS on the device (set_frequency_refactor) in
        the pattern and pivot order of the factors installed now; Yle gives the
        admittance pattern those frequencies share."""
        if tuple(Yle.shape) != (self.n, self.n):
            raise ValueError(f"Yle must be {self.n} x {self.n}")
        yr, yc, _ = self._yle_coo(Yle)
        _lib.check(self.h, self.L.peec_lu_refactor_setup(self.h, int(yr.size), _lib.ptr(yr),
                                                         _lib.ptr(yc)))

    def set_edge_state(self, diagonals, Zs_info, escalings):
        """Uploads the per-edge data from which set_frequency_device forms DZ on the device:
        R and Cd of the four edge halves, the Lp self terms, the real surface-impedance
        base and the surface edges (the inputs of frequency.FrequencyState)."""
        R4 = np.ascontiguousarray(np.real(np.asarray(diagonals["R"])), dtype=np.float64)
        Cd4 = np.ascontiguousarray(np.real(np.asarray(diagonals["Cd"])), dtype=np.float64)
        Lpd = np.ascontiguousarray(np.real(np.asarray(diagonals["Lp"])).ravel(), dtype=np.float64)
        Zs0 = np.ascontiguousarray(np.real(np.asarray(Zs_info["Zs"])).ravel(), dtype=np.float64)
        se = np.ascontiguousarray(np.asarray(Zs_info["surface_edges"]).ravel(), dtype=np.int64)
        if R4.shape != (self.m, 4) or Cd4.shape != (self.m, 4) or Lpd.size != self.m \
                or Zs0.size != self.m:
            raise ValueError(f"edge data must hold {self.m} edges (R and Cd m x 4)")
        _lib.check(self.h, self.L.peec_set_edge_state(
            self.h, _lib.ptr(R4), _lib.ptr(Cd4), _lib.ptr(Lpd), _lib.ptr(Zs0),
            _lib.ptr(se) if se.size else None, int(se.size), float(escalings["R"]),
            float(escalings["freq"])))
        self._edge_state = True

    def set_frequency_device(self, w, Yle, key=None):
        """One frequency's state formed on the device (DZ from the edge data, SS factorised
        in the pattern of enable_refactor); the host passes w and Yle only."""
        if key is not None and self._same_key(key, self._freq_key):
            return
        if tuple(Yle.shape) != (self.n, self.n):
            raise ValueError(f"Yle must be {self.n} x {self.n}")
        yr, yc, yv = self._yle_coo(Yle)
        self._freq_key = None
        _lib.check(self.h, self.L.peec_set_frequency_device(
            self.h, float(w), int(yr.size), _lib.ptr(yr), _lib.ptr(yc),
            _lib.ptr(yv.view(np.float64))))
        self._freq_key = key

    def set_frequency_refactor(self, w, DZ, Yle, key=None):
        """One frequency's state with SS assembled and factorised on the device (after
        enable_refactor); key as for set_frequency."""
        if key is not None and self._same_key(key, self._freq_key):
            return
        DZ = np.ascontiguousarray(np.asarray(DZ, dtype=np.complex128).ravel())
        if DZ.size != self.m:
            raise ValueError(f"DZ has {DZ.size} entries, expected {self.m}")
        if tuple(Yle.shape) != (self.n, self.n):
            raise ValueError(f"Yle must be {self.n} x {self.n}")
        yr, yc, yv = self._yle_coo(Yle)
        self._freq_key = None
        _lib.check(self.h, self.L.peec_set_frequency_refactor(
            self.h, float(w), _lib.ptr(DZ.view(np.float64)), int(yr.size), _lib.ptr(yr),
            _lib.ptr(yc), _lib.ptr(yv.view(np.float64))))
        self._freq_key = key

    # -- operator ----------------------------------------------------------------------
    def matvec(self, x, precision=0):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.complex128).ravel())
        if x.size != self.N:
            raise ValueError(f"x has {x.size} entries, expected {self.N}")
        y = np.empty(self.N, dtype=np.complex128)
        _lib.check(self.h, self.L.peec_matvec(self.h, _lib.ptr(x), _lib.ptr(y), precision))
        return y

    def matvec_dev(self, x_ptr, y_ptr, precision=0):
        _lib.check(self.h, self.L.peec_matvec_dev(self.h, ctypes.c_void_p(x_ptr),
                                                  ctypes.c_void_p(y_ptr), precision))

    def last_timing(self):
        t = [ctypes.c_double() for _ in range(3)]
        self.L.peec_last_timing(self.h, *[ctypes.byref(v) for v in t])
        return tuple(v.value for v in t)

    def stream(self):
        return int(self.L.peec_stream(self.h) or 0)

    def conv_info(self):
        """The six lattice families: circulant grid, extents, presence, kind."""
        out = []
        for i in range(self.L.peec_conv_count(self.h)):
            L = (ctypes.c_int * 3)()
            dims = (ctypes.c_int * 3)()
            active = ctypes.c_int()
            kind = ctypes.c_int()
            _lib.check(self.h, self.L.peec_conv_info(self.h, i, L, dims, ctypes.byref(active),
                                                     ctypes.byref(kind)))
            out.append({"L": tuple(L), "dims": tuple(dims), "active": bool(active.value),
                        "edge": bool(kind.value)})
        return out

    FORMS = ("direct", "direct_yz", "staged")

    def zpass_tuning(self):
        """The FP32 z-pass forms the autotuner picked (face, edge, edge radix plan) and the
        ms it measured per candidate (None where a form was not a candidate)."""
        ch = (ctypes.c_int * 3)()
        fms = np.zeros(3)
        ems = np.zeros(6)
        _lib.check(self.h, self.L.peec_zpass_tuning(self.h, ch, fms.ctypes.data_as(_lib.DP),
                                                    ems.ctypes.data_as(_lib.DP)))
        opt = lambda v: None if v < 0 else float(v)
        return {"face": self.FORMS[ch[0]], "edge": self.FORMS[ch[1]], "edge_plan": int(ch[2]),
                "face_ms": {self.FORMS[i]: opt(fms[i]) for i in range(3)},
                "edge_ms": {f"plan{p_}_{self.FORMS[i]}": opt(ems[3 * p_ + i])
                            for p_ in range(2) for i in range(3)}}

    def set_zpass_forms(self, face, edge, edge_plan=0):
        """Pins the FP32 z-pass forms ("direct", "direct_yz", "staged" or 0..2) in place of
        the tuner's choice until the next fill / set_rows."""
        f = self.FORMS.index(face) if isinstance(face, str) else int(face)
        e = self.FORMS.index(edge) if isinstance(edge, str) else int(edge)
        _lib.check(self.h, self.L.peec_set_zpass_forms(self.h, f, e, int(edge_plan)))

    def profile_matvec(self, precision, iters=10):
        ms = (ctypes.c_double * 7)()
        _lib.check(self.h, self.L.peec_profile_matvec(self.h, int(precision), int(iters), ms))
        keys = ("xfwd", "yfwd", "z", "yinv", "xinv", "sparse", "total")
        return dict(zip(keys, list(ms)))

    def launch_count(self):
        return int(self.L.peec_launch_count(self.h))

    def port_rhs(self, n1, n2, Is):
        tn = np.empty(self.N, dtype=np.complex128)
        _lib.check(self.h, self.L.peec_port_rhs(self.h, int(n1), int(n2), float(Is), _lib.ptr(tn)))
        return tn

    def set_stop_flag(self, flag: "ctypes.c_int | None"):
        self._stop = flag
        _lib.check(self.h, self.L.peec_set_stop_flag(
            self.h, ctypes.cast(ctypes.byref(flag), ctypes.c_void_p) if flag is not None else None))

    def _vectors(self, b, x0):
        b = np.ascontiguousarray(np.asarray(b, dtype=np.complex128).ravel())
        x = np.zeros(self.N, dtype=np.complex128) if x0 is None or np.size(x0) == 0 else \
            np.array(np.asarray(x0, dtype=np.complex128).ravel())
        if b.size != self.N or x.size != self.N:
            raise ValueError(f"b and x0 have {b.size} and {x.size} entries, expected {self.N}")
        return b, x

    def gmres(self, b, x0, tol, maxit, restarted=False, restart=0, precision=0):
        b, x = self._vectors(b, x0)
        flag = ctypes.c_int()
        relres = ctypes.c_double()
        it = (ctypes.c_int * 2)()
        cap = (maxit if not restarted else maxit * max(restart, 1)) + 2
        resvec = np.zeros(cap)
        nres = ctypes.c_int()
        rc = self.L.peec_gmres(self.h, _lib.ptr(b), _lib.ptr(x), float(tol), int(maxit),
                               1 if restarted else 0, int(restart), int(precision),
                               ctypes.byref(flag), ctypes.byref(relres), it,
                               resvec.ctypes.data_as(_lib.DP), cap, ctypes.byref(nres))
        if rc == -3:
            return x, 99, 0.0, [it[0], it[1]], np.zeros(1)
        _lib.check(self.h, rc)
        return x, flag.value, relres.value, [it[0], it[1]], resvec[:nres.value].copy()

    def set_device_loop(self, on: bool):
        """GMRES iterations in a device-resident loop (default) or one host round trip per
        iteration (the same kernels and results)."""
        _lib.check(self.h, self.L.peec_set_device_loop(self.h, 1 if on else 0))

    def device_loop_stats(self):
        """(graph launches, GMRES iterations they ran) since the context was created."""
        a, b = ctypes.c_int64(0), ctypes.c_int64(0)
        _lib.check(self.h, self.L.peec_device_loop_stats(self.h, ctypes.byref(a), ctypes.byref(b)))
        return int(a.value), int(b.value)

    def set_lu_component_max(self, max_rows):
        """Rows of LU components up to max_rows (<= 512) are solved one component per
        warp, the rest by the global synchronisation-free scheme (0, the default: all
        global)."""
        _lib.check(self.h, self.L.peec_set_lu_component_max(self.h, int(max_rows)))

    def adjoint(self, x, v1, v2, d1, d2, Is, nvox):
        """Per-voxel derivative of the port voltage from the port solution x by
        reciprocity (peec_adjoint): (2/Is) * sum over each voxel's edges of
        d1[e] I_e^2 (first voxel v1[e]) or d2[e] I_e^2 (second voxel v2[e])."""
        x = np.ascontiguousarray(np.asarray(x, dtype=np.complex128).ravel())
        if x.size < self.m:
            raise ValueError("x must hold the edge currents first")
        v1 = np.ascontiguousarray(np.asarray(v1, dtype=np.int32).ravel())
        v2 = np.ascontiguousarray(np.asarray(v2, dtype=np.int32).ravel())
        d1 = np.ascontiguousarray(np.asarray(d1, dtype=np.complex128).ravel())
        d2 = np.ascontiguousarray(np.asarray(d2, dtype=np.complex128).ravel())
        if not (v1.size == v2.size == d1.size == d2.size == self.m):
            raise ValueError("v1, v2, d1, d2 need one entry per edge")
        g = np.zeros(int(nvox), dtype=np.complex128)
        _lib.check(self.h, self.L.peec_adjoint(
            self.h, _lib.ptr(x), _lib.ptr(v1), _lib.ptr(v2), _lib.ptr(d1.view(np.float64)),
            _lib.ptr(d2.view(np.float64)), float(Is), int(nvox), _lib.ptr(g.view(np.float64))))
        return g

    def set_residual_precision(self, precision):
        """Arithmetic of the refinement residuals of solve_mixed: PREC_FF (float-float,
        default) or PREC_FP64."""
        _lib.check(self.h, self.L.peec_set_residual_precision(self.h, int(precision)))

    def solve_mixed(self, b, x0, tol, inner_tol=1e-7, inner_maxit=100, max_outer=8):
        b, x = self._vectors(b, x0)
        flag = ctypes.c_int()
        relres = ctypes.c_double()
        outer = ctypes.c_int()
        inner = ctypes.c_int()
        rc = self.L.peec_solve_mixed(
            self.h, _lib.ptr(b), _lib.ptr(x), float(tol), float(inner_tol), int(inner_maxit),
            int(max_outer), ctypes.byref(flag), ctypes.byref(relres), ctypes.byref(outer),
            ctypes.byref(inner))
        if rc == -3:  # cancelled by the stop flag: flag 99, as gmres reports it
            return x, 99, 0.0, 0, 0
        _lib.check(self.h, rc)
        return x, flag.value, relres.value, outer.value, inner.value
