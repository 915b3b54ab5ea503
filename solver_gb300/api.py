"""Drop-in mirrors of the reference's FFT-PEEC entry points, running on the GPU.

Same names, positional arguments and return values as the Julia functions:

* ``compute_FFT_mutual_coupling_mats`` -- compute_FFT_mutual_coupling_mats.jl:1-33
* ``ComputeMatrixVectorFTT``           -- compute_Matrix_vector_fft.jl:1-81
* ``gmres_custom``                     -- gmres_custom.jl:1-331
* ``FFT_solver_QS_S_type``             -- FFT_solver_QS_S_type.jl:1-234

The FFTW plan arguments of the reference (PLIVector, PVector, ...) are accepted
and ignored. The GPU context of a geometry is cached in ``expansions["gpu_ctx"]``,
as a Julia caller would stash it. ``FFTCP`` / ``FFTCLp`` may be the handle this
module returns, or the reference's own 2N-extent spectra (numpy), from which the
generating rows are recovered once on the host.
"""
from __future__ import annotations

import time

import numpy as np

from . import frequency as fq
from .fill_cache import fill_operator
from .operator import GpuOperator, row_dims

_P_KEYS = {(0, 0): "p12_se", (1, 1): "p34_se", (2, 2): "p56_se", (0, 1): "p1234",
           (0, 2): "p1256", (1, 2): "p3456"}
_LP_KEYS = ("Lpx", "Lpy", "Lpz")


class CirculantSpectra:
    """Device-resident spectra of the nine blocks (handle returned as FFTCP and FFTCLp)."""

    def __init__(self, op: GpuOperator, rows: dict | None = None):
        self.op = op
        self.rows = rows


class RccRows(CirculantSpectra):
    """Device-resident quasi-static parts of the nine Rcc rows with their centre distances
    (the handle returned as FFTCP and FFTCLp for QS_Rcc_FW == 2; the reference returns
    the rows_P / rows_Lp dictionaries, compute_FFT_mutual_coupling_mats.jl:17-27). The
    sweep builds the spectra of every frequency from them on the GPU."""


def get_operator(incidence_selection, expansions, diagonals, device=0) -> GpuOperator:
    op = expansions.get("gpu_ctx")
    if op is None or op.h is None:
        op = GpuOperator(incidence_selection, expansions, diagonals["P"], device=device)
        expansions["gpu_ctx"] = op
    return op


def rows_from_reference_spectra(FFTCP, FFTCLp, grid):
    """Generating rows from reference-format spectra: the first octant of the
    inverse FFT of each 2N-extent circulant (store_circulant_fft's inverse)."""
    dims = row_dims(*grid)
    rows = {}
    for c, key in enumerate(_LP_KEYS):
        spec = FFTCLp[c] if not isinstance(FFTCLp[c], (list, tuple)) else FFTCLp[c][0]
        if np.prod(dims[key]) == 0 or spec is None or np.size(spec) == 0:
            continue
        full = np.fft.ifftn(spec)
        d = dims[key]
        rows[key] = np.real(full[:d[0], :d[1], :d[2]]).ravel(order="F")
    for (i, j), key in _P_KEYS.items():
        full = np.fft.ifftn(FFTCP[i][j])
        d = dims[key]
        rows[key] = np.real(full[:d[0], :d[1], :d[2]]).ravel(order="F")
    return rows


def _ensure_spectra(op, FFTCP, FFTCLp):
    if isinstance(FFTCP, RccRows):
        raise ValueError("Rcc rows hold no spectra of their own: the sweep builds them per "
                         "frequency (FFT_solver_QS_S_type with QS_Rcc_FW=2)")
    if isinstance(FFTCP, CirculantSpectra):
        if FFTCP.op is not op:
            raise ValueError("spectra belong to another operator context")
        return
    src = getattr(op, "_spec_src", None)
    if src is not None and src[0] is FFTCP and src[1] is FFTCLp:
        return
    op.set_rows(rows_from_reference_spectra(FFTCP, FFTCLp, op.grid))
    op._spec_src = (FFTCP, FFTCLp)  # held, so these identities stay unique while cached


def compute_FFT_mutual_coupling_mats(circulant_centers, escalings, Nx, Ny, Nz, QS_Rcc_FW=1,
                                     id=None, chan=None, *, incidence_selection=None,
                                     expansions=None, diagonals=None, return_rows=False):
    """GPU fill of the Lp/P generating rows and their spectra. Returns
    (FFTCP, FFTCLp) as one device handle (the reference returns host spectra).
    The operator context is taken from / stored in ``expansions``.
    QS_Rcc_FW == 2: the quasi-static parts of the retarded operator's rows
    (compute_rows_Rcc_P, compute_rows_Rcc_Lp), kept on the device as an RccRows handle."""
    if QS_Rcc_FW not in (1, 2):
        raise NotImplementedError("QS_Rcc_FW must be 1 (quasi-static) or 2 (Rcc); the "
                                  "reference's Taylor variant (3) is commented out")
    op = get_operator(incidence_selection, expansions, diagonals)
    if tuple(op.grid) != (Nx, Ny, Nz):
        raise ValueError("grid does not match the operator's topology")
    if QS_Rcc_FW == 2:
        rows = op.fill_rcc(circulant_centers["origin"], circulant_centers["sx"],
                           circulant_centers["sy"], circulant_centers["sz"], escalings["Lp"],
                           escalings["P"])
        h = RccRows(op, rows if return_rows else None)
        return h, h
    rows = op.fill(circulant_centers["origin"], circulant_centers["sx"], circulant_centers["sy"],
                   circulant_centers["sz"], escalings["Lp"], escalings["P"],
                   return_rows=return_rows)
    h = CirculantSpectra(op, rows)
    return h, h


def _set_freq(op, w, DZ, Yle, lu):
    op.set_frequency(w, DZ, Yle, lu, key=(float(w), DZ, Yle, lu))


def _lu_object(lu):
    # the reference passes the factorisation object; accept scipy SuperLU or
    # a FrequencyState carrying one
    return getattr(lu, "lu", lu)


def ComputeMatrixVectorFTT(x, w, incidence_selection, FFTCP, FFTCLp, DZ, Yle, expansions, invZ,
                           invP, lu, PLIVector=None, PVector=None, PLI2Vector=None, P2Vector=None,
                           chi2Vector=None, *, precision=0, diagonals=None):
    """y = M^-1 K x on the GPU (compute_Matrix_vector_fft.jl:1-81)."""
    op = expansions.get("gpu_ctx")
    if op is None:
        diagP = diagonals["P"] if diagonals is not None else 1.0 / np.asarray(invP.diagonal())
        op = get_operator(incidence_selection, expansions, {"P": diagP})
    _ensure_spectra(op, FFTCP, FFTCLp)
    _set_freq(op, w, DZ, Yle, _lu_object(lu))
    return op.matvec(x, precision)


def gmres_custom(b, restarted, tol, maxit, x, wk, incidence_selection, FFTCP, FFTCLp, DZ, Yle,
                 expansions, invZ, invP, lu, PLIVector=None, PVector=None, PLI2Vector=None,
                 P2Vector=None, chi2Vector=None, id=None, chan=None, portIndex=None, *,
                 restart=None, precision=0, stop_flag=None):
    """Householder GMRES with MATLAB semantics on the GPU (gmres_custom.jl:1-331).
    Returns (x, flag, relres, iter, resvec); flag 99 when stop_flag is set."""
    op = expansions.get("gpu_ctx")
    if op is None:
        op = get_operator(incidence_selection, expansions,
                          {"P": 1.0 / np.asarray(invP.diagonal())})
    _ensure_spectra(op, FFTCP, FFTCLp)
    _set_freq(op, wk, DZ, Yle, _lu_object(lu))
    if stop_flag is not None:
        op.set_stop_flag(stop_flag)
    if restarted and restart is None:
        raise ValueError("restarted GMRES needs an explicit restart length")
    return op.gmres(b, x, tol, maxit, restarted=restarted, restart=restart or 0,
                    precision=precision)


def s2z_fft(S, Zo):
    npt, _, nf = S.shape
    I = np.eye(npt)
    return np.stack([Zo * np.linalg.solve(I - S[:, :, k], I + S[:, :, k]) for k in range(nf)], 2)


def s2y_fft(S, Zo):
    npt, _, nf = S.shape
    I = np.eye(npt)
    return np.stack([Zo * np.linalg.solve(I + S[:, :, k], I - S[:, :, k]) for k in range(nf)], 2)


def install_state(op, fs, device_lu=False):
    """Sets a frequency state on a context: with host factors (fs.lu) through
    peec_set_frequency, and with device_lu the later states factorised on the device in
    their pattern (fs.lu None: peec_set_frequency_refactor); a DeviceFrequencyState has
    its DZ formed on the device too (peec_set_frequency_device)."""
    if getattr(fs, "device_dz", False):
        src = getattr(op, "_edge_src", None)
        if fs.edge is not None and (src is None or src[0] is not fs.edge[0]
                                    or src[1] is not fs.edge[1]):
            # the context's edge data comes from these diagonals (kept referenced, so the
            # identity test cannot match a reused object)
            op.set_edge_state(fs.edge[0], fs.edge[1], fs.escalings)
            op._edge_src = fs.edge
        elif fs.edge is None and not getattr(op, "_edge_state", False):
            raise ValueError("a device-formed state on a context without edge data")
        op.set_frequency_device(fs.w, fs.Yle)
    elif device_lu and fs.lu is None:
        op.set_frequency_refactor(fs.w, fs.DZ, fs.Yle)
    else:
        op.set_frequency(fs.w, fs.DZ, fs.Yle, fs.lu)
        if device_lu:
            op.enable_refactor(fs.Yle)


class PortLanes:
    """Concurrent port solves of one frequency: one context per lane (its own CUDA
    stream, FFT buffers, Krylov workspace and LU-solve control words; same topology
    and circulant rows), each lane driven by its own host thread. The library calls
    release the GIL, so the lanes' kernels overlap on the GPU: the latency-bound
    parts of one port's iteration (triangular solves, small reductions, host round
    trips) fill in around the bandwidth-bound transforms of the others."""

    def __init__(self, op, nlanes):
        from concurrent.futures import ThreadPoolExecutor
        self.ops = [op] + [op.clone() for _ in range(max(1, nlanes) - 1)]
        self._pool = ThreadPoolExecutor(max_workers=len(self.ops))

    def __len__(self):
        return len(self.ops)

    def set_frequency(self, w, DZ, Yle, lu, key=None):
        list(self._pool.map(lambda o: o.set_frequency(w, DZ, Yle, lu, key=key), self.ops))

    def run(self, jobs):
        """jobs[i](op) runs on lane i % lanes; jobs of a lane run in order. Returns the
        results in job order."""
        L = len(self.ops)

        def lane(i):
            return [(j, jobs[j](self.ops[i])) for j in range(i, len(jobs), L)]
        out = [None] * len(jobs)
        for res in self._pool.map(lane, range(L)):
            for j, r in res:
                out[j] = r
        return out

    def sweep(self, seq, get_state, release, pn, Is, Vrest, tol_of, solve_kw, record,
              stop_flag=None, mode="mixed", rcc_hz=None, device_lu=False):
        """Solves of every port at every frequency key of seq, each lane on its own
        through the whole sequence: port c runs on lane c % lanes; a lane sets each
        frequency state on its context, then solves its ports warm-started from its own
        previous solutions (columns of Vrest). No lane waits for another between
        frequencies, so one lane's host work (setting a frequency state, its uploads)
        overlaps the other lanes' GPU solves.

        mode "mixed": peec_solve_mixed with solve_kw (inner_tol, inner_maxit); mode
        "fp64": the reference algorithm, peec_gmres with solve_kw["maxit"].
        get_state(k, pos) -> state with w, DZ, Yle, lu; release(k) is called once every
        lane has set state k. rcc_hz (Rcc operator): k -> Hz; each lane builds that
        frequency's spectra on its own context. device_lu: states without host factors
        (lu None) are factorised on each lane's device in the pattern of the first
        factored state the lane set. record(pos, k, c, V, flag, relres, outer, inner) is called
        from the lane threads after each solve (fp64: outer = 1, inner = the GMRES
        iterations). Returns False if stopped. An exception in one lane stops the others
        before their next frequency or port solve, and is then raised here."""
        if mode not in ("mixed", "fp64"):
            raise ValueError(f"mode must be 'mixed' or 'fp64', not {mode!r}")
        import threading
        L = len(self.ops)
        npt = len(pn)
        left = {}
        lock = threading.Lock()
        stopped = []
        failed = threading.Event()

        def halted():
            return failed.is_set() or (stop_flag is not None and stop_flag.value)

        def lane(i):
            op = self.ops[i]
            mine = range(i, npt, L)
            for pos, k in enumerate(seq):
                if halted():
                    stopped.append(True)
                    return
                fs = get_state(k, pos)
                install_state(op, fs, device_lu)
                if rcc_hz is not None:
                    op.set_rcc_frequency(rcc_hz(k))
                with lock:
                    left[pos] = left.get(pos, min(L, npt)) - 1
                    if left[pos] == 0 and k not in seq[pos + 1:]:
                        release(k)
                for c in mine:
                    if failed.is_set():
                        return
                    tn = op.port_rhs(pn[c][0], pn[c][1], Is)
                    if mode == "mixed":
                        V, flag, relres, outer, inner = op.solve_mixed(tn, Vrest[:, c],
                                                                       tol_of(k), **solve_kw)
                    else:
                        V, flag, relres, it, _ = op.gmres(tn, Vrest[:, c], tol_of(k),
                                                          solve_kw["maxit"])
                        outer, inner = 1, int(it[1])
                    if flag == 99:
                        stopped.append(True)
                        return
                    Vrest[:, c] = V
                    record(pos, k, c, V, flag, relres, outer, inner)

        def guarded_lane(i):
            try:
                lane(i)
            except BaseException:
                failed.set()
                raise

        futs = [self._pool.submit(guarded_lane, i) for i in range(min(L, npt))]
        errors = [f.exception() for f in futs]
        for e in errors:
            if e is not None:
                raise e
        return not stopped

    def close(self):
        self._pool.shutdown(wait=True)
        for o in self.ops[1:]:
            o.close()


# node count from which the per-frequency host factorisations run in worker processes
# (below it, process start-up costs more than the factorisations)
POOL_MIN_NODES = 50000


def FFT_solver_QS_S_type(freq, escalings, incidence_selection, FFTCP, FFTCLp, diagonals, ports,
                         ports_scatter_value, lumped_elements, expansions, GMRES_settings,
                         Zs_info, QS_Rcc_FW=1, id=None, chan=None, commentsEnabled=False, *,
                         mode="fp64", mixed_inner_tol=1e-7, mixed_warm_start=True,
                         stop_flag=None, on_solve=None, lanes=1, records=None, lu="host"):
    """Frequency x port sweep with warm starts (FFT_solver_QS_S_type.jl:1-234).

    mode "fp64": the reference algorithm (FP64 convolutions, Householder GMRES).
    mode "mixed": FP32 convolutions inside FP64 iterative refinement to the same
    relative residual. lanes > 1 (mixed, warm starts): the ports are spread over that
    many contexts (PortLanes), each sweeping its ports through every frequency on its
    own. records: a path; one JSON line per port solve (frequency index and Hz, port,
    mode, flag, relative residual, iterations, wall ms) is appended to it. Returns
    {"S","Z","Y","f","info"}; None if stopped.
    QS_Rcc_FW == 2 (FFTCP / FFTCLp an RccRows handle): the retarded operator, its spectra
    rebuilt on the GPU at every frequency (FFT_solver_QS_S_type.jl:61-93).
    lu "host": SS factorised on the host at every frequency (as the reference does);
    "device": on the host at the first frequency only, then assembled and factorised on
    the GPU in that pattern and pivot order (GpuOperator.set_frequency_refactor).
    """
    if lu not in ("host", "device"):
        raise ValueError(f"lu must be 'host' or 'device', not {lu!r}")
    device_lu = lu == "device"
    factor_of = (lambda k: k == 0) if device_lu else (lambda k: True)
    if QS_Rcc_FW not in (1, 2):
        raise NotImplementedError("QS_Rcc_FW must be 1 (quasi-static) or 2 (Rcc)")
    freq = np.asarray(freq, dtype=np.float64).ravel() * escalings["freq"]
    inner = int(GMRES_settings["Inner_Iter"])
    A = incidence_selection["A"]
    m, n = A.shape
    ns = incidence_selection["Gamma"].shape[1]
    op = get_operator(incidence_selection, expansions, diagonals)
    rcc_hz = None
    if QS_Rcc_FW == 2:
        if not isinstance(FFTCP, RccRows) or FFTCP.op is not op:
            raise ValueError("QS_Rcc_FW == 2 needs the RccRows handle of this operator "
                             "(compute_FFT_mutual_coupling_mats with QS_Rcc_FW=2)")
        # the reference rebuilds at freq[k] / escalings["freq"], the frequency in Hz
        rcc_hz = lambda k: float(freq[k] / escalings["freq"])
    else:
        _ensure_spectra(op, FFTCP, FFTCLp)
    if stop_flag is not None:
        op.set_stop_flag(stop_flag)
    w = 2 * np.pi * freq
    pn = np.asarray(ports["port_nodes"], dtype=np.int64).reshape(-1, 2)
    npt = pn.shape[0]
    S = np.zeros((npt, npt, w.size), dtype=np.complex128)
    Vrest = np.zeros((m + n + ns, npt), dtype=np.complex128)
    tol = GMRES_settings["tol"]
    info = []
    nl = min(int(lanes), npt)
    # lanes read each state once per lane: keep states until every lane has set them
    keep = mode == "mixed" and mixed_warm_start and nl > 1
    if device_lu:
        # the first frequency factorised on the host (its pattern and pivot order); the
        # others formed on the device (DZ, SS and its factors), the host building Yle only
        first = lambda k: fq.FrequencyState(w[k], escalings, incidence_selection, diagonals,
                                            Zs_info, lumped_elements, ports,
                                            ports_scatter_value, factor=True)
        later = lambda k: fq.DeviceFrequencyState(w[k], escalings, n, lumped_elements, ports,
                                                  ports_scatter_value, (diagonals, Zs_info))
        pf = fq.StatePrefetcher(lambda k: first(k) if k == 0 else later(k), range(w.size),
                                keep=keep)
    elif n >= POOL_MIN_NODES and w.size > 2:
        # large node systems: factorise ahead in spawned worker processes
        pf = fq.FrequencyPool((escalings, incidence_selection, diagonals, Zs_info,
                               lumped_elements, ports, ports_scatter_value),
                              lambda k: w[k], range(w.size), workers=4, lookahead=4, keep=keep,
                              factor_of=factor_of)
    else:
        pf = fq.StatePrefetcher(
            lambda k: fq.FrequencyState(w[k], escalings, incidence_selection, diagonals, Zs_info,
                                        lumped_elements, ports, ports_scatter_value,
                                        factor=factor_of(k)),
            range(w.size), keep=keep)
    try:
        if mode == "mixed" and mixed_warm_start and nl > 1:
            res = _sweep_lanes(op, nl, pf, w, pn, S, Vrest, tol, inner, escalings,
                               mixed_inner_tol, stop_flag, on_solve, info, m, ns,
                               ports_scatter_value, rcc_hz, device_lu)
        else:
            res = _sweep(op, pf, w, pn, npt, S, Vrest, tol, inner, escalings, mode,
                         mixed_inner_tol, mixed_warm_start, stop_flag, on_solve, info, m, ns,
                         ports_scatter_value, rcc_hz, device_lu)
    finally:
        pf.close()
    if res is not None:
        res["f"] = freq / escalings["freq"]
        if records is not None:
            _write_records(records, res["info"], res["f"], mode)
    return res


def _write_records(path, info, f_hz, mode):
    import json
    with open(path, "a") as fh:
        for r in info:
            rec = {"freq_index": int(r["freq"]), "f_hz": float(f_hz[r["freq"]]),
                   "port": int(r["port"]), "mode": mode, "flag": int(r["flag"]),
                   "relres": float(r["relres"]), "ms": float(r.get("ms", 0.0))}
            if "iter" in r:
                rec["iterations"] = [int(t) for t in r["iter"]]
            if "outer" in r:
                rec["outer"] = int(r["outer"])
                rec["inner"] = int(r["niter"])
            fh.write(json.dumps(rec) + "\n")


def _port_column(V, pn, c1, m, ns, z0):
    """S entries (c1, c2 >= c1) from port c1's solution (FFT_solver_QS_S_type.jl:199-208)."""
    out = {}
    for c2 in range(c1, len(pn)):
        n3, n4 = pn[c2]
        val = 2 * (V[m + ns + n3] - V[m + ns + n4])
        out[c2] = (val - z0) / z0 if c1 == c2 else val / z0
    return out


def _sweep_lanes(op, nl, pf, w, pn, S, Vrest, tol, inner, escalings, mixed_inner_tol,
                 stop_flag, on_solve, info, m, ns, z0, rcc_hz=None, device_lu=False):
    lanes = PortLanes(op, nl)
    if stop_flag is not None:
        for o in lanes.ops[1:]:
            o.set_stop_flag(stop_flag)
    recs = []
    lock = __import__("threading").Lock()

    def record(pos, k, c1, V, flag, relres, outer, ninner):
        col = _port_column(V, pn, c1, m, ns, z0)
        with lock:
            recs.append(({"flag": flag, "relres": relres, "outer": outer, "niter": ninner,
                          "freq": k, "port": c1}, col))
            if on_solve:
                on_solve(k, c1, V)

    try:
        ok = lanes.sweep(list(range(w.size)), pf.get, pf.release, pn, escalings["Is"], Vrest,
                         lambda k: float(tol[k]) if np.ndim(tol) else float(tol),
                         dict(inner_tol=mixed_inner_tol, inner_maxit=inner), record,
                         stop_flag=stop_flag, rcc_hz=rcc_hz, device_lu=device_lu)
    finally:
        lanes.close()
    if not ok:
        return None
    recs.sort(key=lambda r: (r[0]["freq"], r[0]["port"]))
    for rec, col in recs:
        k, c1 = rec["freq"], rec["port"]
        for c2, v in col.items():
            S[c1, c2, k] = v
            S[c2, c1, k] = v
        info.append(rec)
    return {"S": S, "Z": s2z_fft(S, z0), "Y": s2y_fft(S, z0), "info": info, "Vrest": Vrest}


def _sweep(op, pf, w, pn, npt, S, Vrest, tol, inner, escalings, mode, mixed_inner_tol,
           mixed_warm_start, stop_flag, on_solve, info, m, ns, ports_scatter_value,
           rcc_hz=None, device_lu=False):
    for k in range(w.size):
        if stop_flag is not None and stop_flag.value:
            return None
        fs = pf.get(k)
        install_state(op, fs, device_lu)
        if rcc_hz is not None:
            op.set_rcc_frequency(rcc_hz(k))
        tk = float(tol[k]) if np.ndim(tol) else float(tol)
        for c1 in range(npt):
            n1, n2 = pn[c1]
            tn = op.port_rhs(n1, n2, escalings["Is"])
            t0 = time.perf_counter()
            if mode == "fp64":
                V, flag, relres, it, resvec = op.gmres(tn, Vrest[:, c1], tk, inner)
                rec = {"flag": flag, "relres": relres, "iter": it, "niter": len(resvec) - 1}
            elif mode == "mixed":
                x0 = Vrest[:, c1] if mixed_warm_start else np.zeros_like(Vrest[:, c1])
                V, flag, relres, outer, ninner = op.solve_mixed(tn, x0, tk,
                                                                inner_tol=mixed_inner_tol,
                                                                inner_maxit=inner)
                rec = {"flag": flag, "relres": relres, "outer": outer, "niter": ninner}
            else:
                raise ValueError(mode)
            if flag == 99:
                return None
            rec.update(freq=k, port=c1, ms=(time.perf_counter() - t0) * 1e3)
            info.append(rec)
            if on_solve:
                on_solve(k, c1, V)
            Vrest[:, c1] = V
            for c2 in range(c1, npt):
                n3, n4 = pn[c2]
                val = 2 * (V[m + ns + n3] - V[m + ns + n4])
                if c1 == c2:
                    S[c1, c2, k] = (val - ports_scatter_value) / ports_scatter_value
                else:
                    S[c1, c2, k] = val / ports_scatter_value
                    S[c2, c1, k] = S[c1, c2, k]
    return {"S": S, "Z": s2z_fft(S, ports_scatter_value), "Y": s2y_fft(S, ports_scatter_value),
            "info": info, "Vrest": Vrest}


def dump_json_data(matrix_Z, matrix_S, matrix_Y, num_ports, id, partial=False, freqIndex=None):
    """The results dictionary of the reference (format_input_output_solver_functions.jl:
    1-31): per port pair (i outer, j inner) a list holding the per-frequency [re, im]
    pairs, each matrix serialised as a JSON string."""
    import json

    def enc(M):
        M = np.asarray(M, dtype=np.complex128)
        return json.dumps([[[[float(v.real), float(v.imag)] for v in M[i, j, :]]]
                           for i in range(num_ports) for j in range(num_ports)])

    return {"matrices": {"matrix_Z": enc(matrix_Z), "matrix_S": enc(matrix_S),
                         "matrix_Y": enc(matrix_Y)},
            "isStopped": False, "id": id, "partial": partial, "freqIndex": freqIndex}


def do_solving_fft(request, id="job", mode="mixed", lanes=1, device=0, stop_flag=None,
                   records=None, row_cache=None, lu="host"):
    """A solve request end to end, as the reference's doSolvingFFT does it
    (do_solving_fft.jl:1-177) without its message queue and object store: the request
    body (mesherOutput / solverInput / solverAlgoParams / solverType) through the mesher,
    the GPU fill and the frequency x port sweep. Returns the reference's results
    dictionary (dump_json_data) plus "S", "Z", "Y" (ports x ports x frequencies) and
    "f"; None if stopped. mode "fp64" runs the reference algorithm, "mixed" the mixed
    precision solves (lanes: port lanes, see FFT_solver_QS_S_type). row_cache: a
    fill_cache.RowCache, to reuse the rows of an earlier fill of the same lattice. lu: where
    SS is factorised after the first frequency (see FFT_solver_QS_S_type)."""
    from . import mesher
    solver_type = int(request.get("solverType", 1))
    if solver_type not in (1, 2):
        raise NotImplementedError("solverType must be 1 (quasi-static) or 2 (Rcc); the "
                                  "reference's Taylor variant (3) is commented out")
    out, freqs, settings, z0, grid = mesher.parse_request(request, device=device)
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    op = GpuOperator(inc, exp, diag["P"], device=device)
    try:
        if solver_type == 2:
            op.fill_rcc(cc["origin"], cc["sx"], cc["sy"], cc["sz"], esc["Lp"], esc["P"])
            h = RccRows(op)
        else:
            fill_operator(op, cc, esc, row_cache)
            h = CirculantSpectra(op)
        exp["gpu_ctx"] = op
        st = {"Inner_Iter": settings["Inner_Iter"],
              "tol": np.full(len(freqs), settings["tol"])}
        res = FFT_solver_QS_S_type(freqs, esc, inc, h, h, diag, ports, z0, le, exp, st, Zs,
                                   QS_Rcc_FW=solver_type, mode=mode, lanes=lanes,
                                   stop_flag=stop_flag, records=records, lu=lu)
    finally:
        exp.pop("gpu_ctx", None)
        op.close()
    if res is None:
        return None
    npt = res["S"].shape[0]
    outd = dump_json_data(res["Z"], res["S"], res["Y"], npt, id)
    outd.update(S=res["S"], Z=res["Z"], Y=res["Y"], f=res["f"], info=res["info"])
    return outd


def sweep_many(requests, mode="mixed", concurrency=4, device=0, row_cache=None, lu="host"):
    """Frequency sweeps of several geometries, concurrently: each geometry gets its own
    context (CUDA stream, fill, spectra, workspaces) and host thread, so the sweeps' kernels
    overlap on the GPU the way port lanes do. Per request: the mesher, the GPU fill, then
    FFT_solver_QS_S_type in the given mode. Returns the results in request order.
    row_cache: a fill_cache.RowCache; geometries on the same lattice then fill once."""
    from concurrent.futures import ThreadPoolExecutor
    from . import mesher
    from .operator import GpuOperator

    def one(req):
        out, freqs, settings, z0, grid = mesher.parse_request(req, device=device)
        esc, inc, cc, diag, exp, ports, le, li, Zs = out
        op = GpuOperator(inc, exp, diag["P"], device=device)
        try:
            fill_operator(op, cc, esc, row_cache)
            exp["gpu_ctx"] = op
            h = CirculantSpectra(op)
            st = {"Inner_Iter": settings["Inner_Iter"],
                  "tol": np.full(len(freqs), settings["tol"])}
            return FFT_solver_QS_S_type(freqs, esc, inc, h, h, diag, ports, z0, le, exp, st, Zs,
                                        mode=mode, lu=lu)
        finally:
            exp.pop("gpu_ctx", None)
            op.close()

    with ThreadPoolExecutor(max_workers=max(1, concurrency)) as pool:
        return list(pool.map(one, requests))
