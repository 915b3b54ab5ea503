"""Per-frequency host setup of the operator (FFT_solver_QS_S_type.jl:105-119).

Builds, for scaled angular frequency w, the diagonal DZ, the termination/lumped
admittance Yle, and the sparse LU factorisation of the node Schur complement
    SS = Yle + A' diag(1/DZ) A + jw Gamma diag(1/P) Gamma'
on the host (SuperLU via scipy), as the reference factorises with UMFPACK on the host.
The factors are exported in the CSR form the GPU triangular solves consume.
"""
from __future__ import annotations

import math

import threading

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def z_self(R, Cd, w):
    """Sum over the four edge halves of 1/(1/R + jwCd) (compute_Z_self.jl:1-15)."""
    Z = np.zeros(R.shape[0], dtype=np.complex128)
    for aux in range(4):
        r, cd = R[:, aux], Cd[:, aux]
        rc = (r != 0) & (cd != 0)
        ro = (r != 0) & (cd == 0)
        co = (r == 0) & (cd != 0)
        Z[rc] += 1.0 / (1.0 / r[rc] + 1j * w * cd[rc])
        Z[ro] += r[ro]
        Z[co] += 1.0 / (1j * w * cd[co])
    return Z


def _bad(y):
    return not np.isfinite(y) or abs(y) < 1e-16


# Admittance of each lumped element type as a cascade of networks: the first is the
# element itself; while the value is not finite or below 1e-16 in magnitude, the next
# (a network with a vanishing R, L or C dropped) is taken (build_Yle_FFT.jl:128-209).
# Types: 1 series R-L-C, 2 (R + L) parallel C, 3 (R + C) parallel L, 4 R | C | L in
# parallel, 5 R parallel (L + C). Divisions by zero follow IEEE arithmetic, as in Julia.
_CASCADES = {
    2: (lambda R, L, C, jw: 1 / (R + jw * L) + jw * C,
        lambda R, L, C, jw: 1 / R + jw * C,
        lambda R, L, C, jw: 1 / (R + jw * L),
        lambda R, L, C, jw: 1 / R,
        lambda R, L, C, jw: 1 / (jw * L) + jw * C,
        lambda R, L, C, jw: jw * C),
    3: (lambda R, L, C, jw: 1 / (R + 1 / (jw * C)) + 1 / (jw * L),
        lambda R, L, C, jw: 1 / (R + 1 / (jw * C)),
        lambda R, L, C, jw: 1 / R + 1 / (jw * L),
        lambda R, L, C, jw: 1 / R,
        lambda R, L, C, jw: 1 / (1 / (jw * C)) + 1 / (jw * L),
        lambda R, L, C, jw: 1 / (jw * L),
        lambda R, L, C, jw: 1 / (1 / (jw * C))),
    4: (lambda R, L, C, jw: 1 / R + jw * C + 1 / (jw * L),
        lambda R, L, C, jw: 1 / R + jw * C,
        lambda R, L, C, jw: jw * C + 1 / (jw * L),
        lambda R, L, C, jw: jw * C),
    5: (lambda R, L, C, jw: 1 / R + 1 / (jw * L + 1 / (jw * C)),
        lambda R, L, C, jw: 1 / R + 1 / (1 / (jw * C)),
        lambda R, L, C, jw: 1 / R + 1 / (jw * L),
        lambda R, L, C, jw: 1 / R,
        lambda R, L, C, jw: 1 / (jw * L + 1 / (jw * C)),
        lambda R, L, C, jw: 1 / (jw * L),
        lambda R, L, C, jw: 1 / (1 / (jw * C))),
}


def lumped_admittance(typ, R, L, C, w):
    """Admittance of a lumped element of type 1..5 at angular frequency w
    (build_Yle_FFT.jl:128-209); 0 where no network of the type is finite."""
    R, L, C = np.float64(R), np.float64(L), np.float64(C)
    jw = np.complex128(1j * w)
    with np.errstate(all="ignore"):
        if typ == 1:
            z = R + jw * L + 1 / (jw * C)
            if _bad(z):
                z = R + jw * L
            y = 1 / z
        elif typ in _CASCADES:
            steps = _CASCADES[typ]
            y = steps[0](R, L, C, jw)
            for step in steps[1:]:
                if not _bad(y):
                    break
                y = step(R, L, C, jw)
        else:
            raise ValueError(f"lumped element type {typ} is not one of 1..5")
    return complex(y) if np.isfinite(y) else 0.0


def yle_matrix(lumped_elements, ports, n, w_real, z0, escal_yle):
    """Sparse n x n admittance of port terminations (1/Z0) and lumped elements
    (build_Yle_FFT.jl:1-126), escaled."""
    rows, cols, vals = [], [], []

    def stamp(a, b, y):
        rows.extend((a, b, a, b))
        cols.extend((a, b, b, a))
        vals.extend((y, y, -y, -y))

    le = lumped_elements
    for k in range(len(le.get("le_nodes", []))):
        y = lumped_admittance(int(le["type"][k]), float(le["R_value"][k]), float(le["L_value"][k]),
                              float(le["C_value"][k]), w_real)
        stamp(int(le["le_nodes"][k][0]), int(le["le_nodes"][k][1]), y)
    for a, b in np.asarray(ports["port_nodes"], dtype=np.int64):
        stamp(int(a), int(b), 1.0 / z0)
    return sp.coo_matrix((np.asarray(vals, dtype=np.complex128) * escal_yle, (rows, cols)),
                         shape=(n, n)).tocsr()


class FrequencyState:
    """DZ, Yle and the factorised SS at one frequency (the reference factorises with
    UMFPACK, FFT_solver_QS_S_type.jl:119; any sparse LU of SS gives the same operator)."""

    def __init__(self, w, escalings, incidence_selection, diagonals, Zs_info, lumped_elements,
                 ports, z0, DZ=None, factor=True):
        """DZ (optional) replaces the edge impedances built from diagonals and Zs_info
        (per-voxel conductivities, see gradient.dz_edges). factor=False skips the host
        factorisation (lu None): the state of a frequency the device factorises
        (GpuOperator.set_frequency_refactor)."""
        A = incidence_selection["A"]
        Gamma = incidence_selection["Gamma"]
        n = A.shape[1]
        self.w = w
        self.Yle = yle_matrix(lumped_elements, ports, n, w / escalings["freq"], z0,
                              escalings["Yle"])
        Zself = z_self(diagonals["R"], diagonals["Cd"], w)
        Zs = escalings["R"] * (np.asarray(Zs_info["Zs"]).ravel() * math.sqrt(w / escalings["freq"]))
        se = np.asarray(Zs_info["surface_edges"], dtype=np.int64)
        d = Zs[se].real - Zself[se].real
        Zself[se[d > 0]] = 1j * Zself[se[d > 0]].imag
        Zs = Zs.copy()
        Zs[se[d < 0]] = 1j * Zs[se[d < 0]].imag
        self.DZ = Zself + Zs.real + 1j * w * np.asarray(diagonals["Lp"]).ravel()
        if DZ is not None:
            self.DZ = np.asarray(DZ, dtype=np.complex128).ravel()
        self.invZ = sp.diags(1.0 / self.DZ)
        self.invP = sp.diags(1.0 / np.asarray(diagonals["P"]).ravel())
        self.SS = self.lu = None
        if not factor:
            return
        SS = (self.Yle + A.T @ (self.invZ @ A) + 1j * w * ((Gamma @ self.invP) @ Gamma.T)).tocsc()
        self.SS = SS
        # SS is structurally symmetric: minimum degree on A'+A keeps the fill of COLAMD
        # and gives shallower elimination trees (fewer dependent levels in the GPU
        # triangular solves)
        self.lu = spla.splu(SS, permc_spec="MMD_AT_PLUS_A", options={"Equil": False})


class DeviceFrequencyState:
    """A frequency state whose edge impedances DZ the device forms (GpuOperator.
    set_frequency_device, after set_edge_state and enable_refactor): the host builds only
    the termination / lumped admittance Yle, microseconds of work."""

    device_dz = True

    def __init__(self, w, escalings, n, lumped_elements, ports, z0, edge=None):
        """edge: (diagonals, Zs_info), uploaded to a context that lacks its edge data when
        the state is installed (api.install_state)."""
        self.w = w
        self.Yle = yle_matrix(lumped_elements, ports, n, w / escalings["freq"], z0,
                              escalings["Yle"])
        self.DZ = None
        self.lu = None
        self.edge = edge
        self.escalings = escalings


class ExportedLU:
    """Factors already in the exported CSR form (picklable, unlike a SuperLU object)."""

    def __init__(self, parts):
        self.parts = parts


def export_lu(lu):
    """CSR factors and permutations with Pr*SS*Pc = L*U from a SuperLU object."""
    if isinstance(lu, ExportedLU):
        return lu.parts
    L = lu.L.tocsr()
    U = lu.U.tocsr()
    L.sort_indices()
    U.sort_indices()

    def parts(M):
        return (M.indptr.astype(np.int64), M.indices.astype(np.int64),
                np.ascontiguousarray(M.data.astype(np.complex128)).view(np.float64))

    return parts(L), parts(U), lu.perm_r.astype(np.int64), lu.perm_c.astype(np.int64)


class StatePrefetcher:
    """Frequency-loop pipelining: while the GPU solves frequency k, a worker thread
    builds the host state (Yle, SuperLU factors) of the next frequency in the
    sequence. The GPU solves run inside foreign calls that release the GIL, so the
    factorisation proceeds alongside them.

    make(k) -> state; order: the sequence of k the caller will request; keep: hold
    every built state for repeated requests (otherwise a state is dropped once read)."""

    def __init__(self, make, order, keep=True):
        from concurrent.futures import ThreadPoolExecutor
        self._make = make
        self._order = list(order)
        self._pos = 0
        self._pool = ThreadPoolExecutor(max_workers=1)
        self._pending = {}
        self._done = {}
        self._keep = keep
        self._lock = threading.Lock()

    def get(self, k, pos=None):
        """The state of key k. pos, the caller's index in the sequence, sets which state
        is started next (callers that walk the sequence concurrently pass it); without
        it the position advances to the next occurrence of k."""
        with self._lock:
            if k in self._done:
                fut, st = None, self._done[k]
            elif k in self._pending:
                fut = self._pending[k]
            else:
                fut = self._pending[k] = self._pool.submit(self._make, k)
            if pos is None:
                while self._pos < len(self._order) and self._order[self._pos] != k:
                    self._pos += 1
                pos = self._pos
                self._pos += 1
            nxt = self._order[pos + 1] if pos + 1 < len(self._order) else None
            if nxt is not None and nxt not in self._done and nxt not in self._pending:
                self._pending[nxt] = self._pool.submit(self._make, nxt)
        if fut is not None:
            st = fut.result()
            with self._lock:
                if self._pending.get(k) is fut:
                    del self._pending[k]
                    if self._keep:
                        self._done[k] = st
        return st

    def release(self, k):
        """Drops a kept state."""
        with self._lock:
            self._done.pop(k, None)

    def close(self):
        self._pool.shutdown(wait=True)


class HostFrequency:
    """Per-frequency host state in picklable form: w, DZ, Yle and the exported LU."""

    def __init__(self, w, DZ, Yle, lu_parts):
        self.w = w
        self.DZ = DZ
        self.Yle = Yle
        self.lu = ExportedLU(lu_parts) if lu_parts is not None else None


_worker_static = None


def _worker_init(static):
    global _worker_static
    _worker_static = static


def _worker_state(w, factor=True):
    fs = FrequencyState(w, *_worker_static, factor=factor)
    return HostFrequency(w, fs.DZ, fs.Yle, export_lu(fs.lu) if factor else None)


class FrequencyPool:
    """Frequency-loop pipelining across processes: spawned workers build the host
    states (Yle, SuperLU factorisation, exported factors) of the next `lookahead`
    frequencies of the sequence while the GPU solves the current one. SuperLU holds
    the GIL for its allocations, so threads would serialise; processes do not.

    static: (escalings, incidence_selection, diagonals, Zs_info, lumped_elements,
    ports, z0), sent to each worker once; w_of(k) the angular frequency of key k;
    factor_of(k) (default: always) whether key k's state carries host factors."""

    def __init__(self, static, w_of, order, workers=4, lookahead=4, keep=True, executor=None,
                 factor_of=None):
        self._own = executor is None
        self._pool = FrequencyPool.executor(static, workers) if executor is None else executor
        self._w_of = w_of
        self._order = list(order)
        self._pos = 0
        self._ahead = max(1, lookahead)
        self._pending = {}
        self._done = {}
        self._keep = keep
        self._lock = threading.Lock()
        # key -> whether its state needs host factors (False: the device factorises)
        self._factor_of = factor_of or (lambda k: True)

    @staticmethod
    def executor(static, workers):
        """The spawned worker processes, each holding `static`. Several pools (for
        example one per walk of a frequency sequence) can share one executor, so that
        the workers are started and their imports paid only once."""
        import multiprocessing
        from concurrent.futures import ProcessPoolExecutor
        return ProcessPoolExecutor(max_workers=workers,
                                   mp_context=multiprocessing.get_context("spawn"),
                                   initializer=_worker_init, initargs=(static,))

    def _submit(self, k):
        if k not in self._done and k not in self._pending:
            self._pending[k] = self._pool.submit(_worker_state, self._w_of(k),
                                                 bool(self._factor_of(k)))

    def get(self, k, pos=None):
        """The state of key k (blocking until a worker has built it). pos, the caller's
        index in the sequence, sets which states are started ahead (callers that walk
        the sequence concurrently pass it); without it the position advances to the
        next occurrence of k. Safe to call from several threads."""
        with self._lock:
            if pos is None:
                while self._pos < len(self._order) and self._order[self._pos] != k:
                    self._pos += 1
                pos = self._pos
                self._pos += 1
            for nxt in self._order[pos:pos + 1 + self._ahead]:
                self._submit(nxt)
            if k in self._done:
                return self._done[k]
            self._submit(k)
            fut = self._pending[k]
        st = fut.result()
        with self._lock:
            if self._pending.get(k) is fut:
                del self._pending[k]
                if self._keep:
                    self._done[k] = st
        return st

    def release(self, k):
        """Drops a kept state."""
        with self._lock:
            self._done.pop(k, None)

    def close(self):
        """Cancels what was not started; shuts the workers down if this pool started
        them (a shared executor stays up for its owner)."""
        for f in self._pending.values():
            f.cancel()
        if self._own:
            self._pool.shutdown(wait=True)
