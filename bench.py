#!/usr/bin/env python
"""Benchmark of the GB300 FFT-PEEC solver path.

Metric: frequency-point solves per second at 1e-8 relative (left-preconditioned)
residual on the 128x128x64 synthetic voxel geometry (Bernoulli(0.3) occupancy,
copper / dielectric 50/50, 4 ports, 10 frequencies 10 MHz-10 GHz). One step = one
frequency point: that frequency's state (DZ, Yle, the factorised SS), then for each of
the 4 ports its right-hand side and a solve warm started from the previous
frequency's solution (FFT_solver_QS_S_type.jl:60-209).

* value: device throughput of the mixed-precision path (FP32 circulant
  convolutions inside iterative refinement) on 4 port lanes -- CUDA events spanning
  the lanes' streams around the GPU part of each step (frequency state, SS
  factorisation on the GPU with --lu device, 4 port solves), the host parts of the
  states prepared beforehand;
* e2e: the same steps end to end through the public API with host buffers, wall clock
  including each point's state built inside the timed region (with --lu device: Yle on
  the host, DZ and the factorisation of SS on the GPU; with --lu host: worker processes
  building DZ, Yle and the SuperLU factors), uploads and the download of each solution;
* fp64_plain: the reference algorithm (FP64 convolutions, Householder GMRES) on the
  same lanes and points; mixed_fp64_residual: mixed with FP64 refinement residuals;
* accuracy: port impedances of every arm against FP64 GMRES at 1e-12, per frequency;
* roofline: the z passes of the FP32 convolutions (forward FFT, 3x3 spectral
  product, inverse FFT), algorithmic bytes from the family descriptors, duration from
  CUDA events around the pass;
* cpu_baseline: the CPU oracle restatement (reference 2N extents, scipy FFT on all
  host cores, SuperLU) timed on complete port solves.

Multi-GPU: the path does not shard; --gpus N runs N independent replicas
(torchrun, one rank per GPU) and reports their summed throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "freq-point solves/s at 1e-8 residual, mixed vs FP64 plain on 1 GB300; matvec GB/s"
UNIT = "freq-point solves/s"
WORKLOAD = ("random_128x128x64: 5e-5 m voxels, Bernoulli(0.3) occupancy (seed 2), Cu/dielectric "
            "50/50, 4 ports, 10 freqs 10 MHz-10 GHz, tol 1e-8")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=7)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=7,
                    help="timed FP64-plain points (the first of the mixed run's timed points)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--adjoint", action="store_true",
                    help="run the adjoint-gradient configuration instead")
    ap.add_argument("--batched-sweep", action="store_true",
                    help="run the batched multi-geometry sweep configuration instead")
    ap.add_argument("--ris", action="store_true",
                    help="run the dense RIS solver configuration instead")
    ap.add_argument("--reuse-fills", action="store_true",
                    help="batched sweep: geometries on the same lattice share one fill "
                         "(fill_cache.RowCache)")
    ap.add_argument("--small-configs", action="store_true",
                    help="the crossbar 20x20x4 configurations (FP64 plain and mixed per "
                         "frequency), one JSON line")
    ap.add_argument("--profile-only", action="store_true",
                    help="set up, time the operator applications and exit (for ncu captures)")
    ap.add_argument("--host-states", choices=["processes", "thread"], default="processes",
                    help="where the per-frequency host states (SuperLU) are built: spawned "
                         "worker processes (default) or one worker thread")
    ap.add_argument("--lu", choices=["device", "host"], default="device",
                    help="where SS is factorised at the timed frequencies: on the GPU in the "
                         "pattern of one host factorisation made in the warm-up (device), or "
                         "by SuperLU on the host at every frequency (host)")
    ap.add_argument("--krylov-loop", choices=["device", "host"], default="device",
                    help="GMRES iterations in the device-resident loop (a CUDA graph with a "
                         "WHILE node) or one host round trip per iteration (same kernels)")
    ap.add_argument("--lu-solve", choices=["groups", "global"], default="groups",
                    help="LU solves per warp group of factor components (groups) or by the "
                         "synchronisation-free global scheme alone (global)")
    ap.add_argument("--lanes", type=int, default=4,
                    help="concurrent port solves (contexts + host threads), at most the ports")
    ap.add_argument("--inner-tol", type=float, default=1e-7,
                    help="floor of the inner FP32 GMRES relative tolerance")
    ap.add_argument("--profile-iters", type=int, default=20)
    ap.add_argument("--ref-budget", type=float, default=150.0,
                    help="reference arm: seconds of port solves after which no new solve starts")
    ap.add_argument("--grid", type=int, nargs=3, default=None,
                    help="smaller random Cu/dielectric grid (profiling captures and tests only)")
    return ap.parse_args()


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return ws, rank, local


def barrier_max(ws, value):
    """The maximum of value over the ranks (a device tensor under NCCL, a host tensor
    under gloo)."""
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rates(ws, steps, gpu_s, wall_s):
    """Replicas: every rank solves `steps` frequency points of its own. The whole-job rate
    is the points of all ranks over the slowest rank's time, for the device-timed value
    and for the end-to-end wall clock."""
    gpu_max = barrier_max(ws, gpu_s)
    wall_max = barrier_max(ws, wall_s)
    return ws * steps / gpu_max, ws * steps / wall_max, gpu_max, wall_max


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={device}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


def conv_bytes(info, prec, staged=None):
    """Algorithmic bytes of the convolution passes per operator application: every
    per-family intermediate written once and read once by the next pass, each
    spectrum read once, lattice maps (int32) once, compact vectors (complex128) read
    once by the gather and written once by the scatter. Spectra: full form (face
    families: 3 real + 3 complex on the shared grid; edge families: one real each), or
    for the staged FP32 z passes (staged = {"faces", "edges"}) the y/z-folded real
    tables of Lx(Ly/2+1)(Lz/2+1) floats (six for the faces, one per edge family)."""
    c = 16 if prec == 0 else 8
    staged = staged or {"faces": False, "edges": False}
    b = {"xfwd": 0, "yfwd": 0, "z": 0, "yinv": 0, "xinv": 0}
    for f in info:
        if not f["active"]:
            continue
        Lx, Ly, Lz = f["L"]
        nx, ny, nz = f["dims"]
        cells = nx * ny * nz
        t_x = Lx * ny * nz * c          # after / before the x pass
        t_y = Lx * Ly * nz * c          # after / before the y pass
        b["xfwd"] += cells * 4 + cells * 16 + t_x
        b["yfwd"] += t_x + t_y
        b["z"] += 2 * t_y
        b["yinv"] += t_y + t_x
        b["xinv"] += t_x + cells * 4 + cells * 16
        G = Lx * Ly * Lz
        folded = Lx * (Ly // 2 + 1) * (Lz // 2 + 1) * 4
        if prec == 1 and staged["edges" if f["edge"] else "faces"]:
            b["z"] += folded if f["edge"] else 2 * folded  # per face family: 2 of the 6 tables
        else:
            b["z"] += (G * c // 2) if f["edge"] else (G * c // 2 + G * c)  # per face family: 1 real + 1 complex
    return b
def reference_model_bytes(grid, c):
    """Bytes per operator application under the pruned three-pass pencil model counted at
    the reference's own circulant extents (4.25 complex elements per padded point per
    block application, cross P blocks applied twice): the work the reference's FFT
    scheme moves, for an effective-bandwidth comparison."""
    Nx, Ny, Nz = grid
    ext = [(2 * (Nx - 1), 2 * Ny, 2 * Nz), (2 * Nx, 2 * (Ny - 1), 2 * Nz),
           (2 * Nx, 2 * Ny, 2 * (Nz - 1)), (2 * Nx, 2 * (Ny + 1), 2 * Nz),
           (2 * (Nx + 1), 2 * Ny, 2 * Nz), (2 * Nx, 2 * Ny, 2 * (Nz + 1))]
    cross = [(2 * (2 * Nx + 1), 2 * (2 * Ny + 1), 2 * Nz), (2 * Nx, 2 * (2 * Ny + 1), 2 * (2 * Nz + 1)),
             (2 * (2 * Nx + 1), 2 * Ny, 2 * (2 * Nz + 1))]
    G = sum(a * b * d for a, b, d in ext) + 2 * sum(a * b * d for a, b, d in cross)
    return 4.25 * G * c


def conv_gbs(b, prof):
    keys = ("xfwd", "yfwd", "z", "yinv", "xinv")
    return sum(b[k] for k in keys) / (sum(prof[k] for k in keys) * 1e-3) / 1e9


# the FP32 z-pass kernels of each tuner form
ZKERNEL = {"face": {"direct": "k_zconv3<float>", "direct_yz": "k_zconv3_yz",
                    "staged": "k_zconv3_staged"},
           "edge": {"direct": "k_zconv1<float> x3", "direct_yz": "k_zconv1_yz x3",
                    "staged": "k_zedge_staged"}}


def z_traffic(grid, tuning):
    """DRAM bytes (read + write) of one operator application's FP32 z passes, as captured
    by ncu for these kernel forms on this grid and recorded in profiles/dram_traffic.json
    (keyed "<face form>+<edge form>"); None when no such capture is recorded."""
    form = f"{tuning['face']}+{tuning['edge']}"
    try:
        d = json.loads((ROOT / "profiles" / "dram_traffic.json").read_text())
        return d["z_passes_fp32"][form].get("x".join(str(int(g)) for g in grid))
    except (OSError, ValueError, KeyError):
        return None


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def setup_problem(device=0, grid=None):
    from solver_gb300 import configs, mesher
    from solver_gb300.operator import GpuOperator
    req = configs.random_128x128x64() if grid is None else configs.random_mixed(tuple(grid))
    out, freqs, settings, z0, grid = mesher.parse_request(req, device=device)
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    op = GpuOperator(inc, exp, diag["P"], device=device)
    rows = op.fill(cc["origin"], cc["sx"], cc["sy"], cc["sz"], esc["Lp"], esc["P"],
                   return_rows=True)
    # the fill again, timed: nine generating rows on the GPU plus their spectra
    t = time.perf_counter()
    op.fill(cc["origin"], cc["sx"], cc["sy"], cc["sz"], esc["Lp"], esc["P"])
    fill_s = time.perf_counter() - t
    return dict(req=req, esc=esc, inc=inc, cc=cc, diag=diag, exp=exp, ports=ports, le=le,
                Zs=Zs, freqs=freqs, settings=settings, z0=z0, grid=grid, op=op, rows=rows,
                fill_s=fill_s)


def fill_report(P, with_cpu):
    """Fill throughput: row entries per second of the GPU fill (rows and spectra), and of
    the oracle's C fill with OpenMP on every host core (the cpu_baseline leg, on the
    oracle mesher's lattice centres; its rows are kept for the CPU solve sample)."""
    entries = int(sum(np.asarray(r).size for r in P["rows"].values()))
    out = {"entries": entries, "gpu_ms": P["fill_s"] * 1e3,
           "gpu_entries_per_s": entries / P["fill_s"]}
    if with_cpu:
        from oracle import mesher_ref as OM
        from oracle import peec_oracle as O
        t = time.perf_counter()
        P["oracle"] = OM.parse_request(P["req"])
        out["cpu_mesh_ms"] = (time.perf_counter() - t) * 1e3
        (esc, inc, cc, *_r), _f, _s, _z, grid = P["oracle"]
        t = time.perf_counter()
        P["oracle_rows"] = O.fill_rows(cc, esc, *grid)
        cpu_s = time.perf_counter() - t
        out.update(cpu_ms=cpu_s * 1e3, cpu_entries_per_s=entries / cpu_s,
                   cpu_cores=os.cpu_count() or 1, cpu_kind="port")
    return out


def freq_state(P, k, factor=True):
    from solver_gb300 import frequency as fq
    w = 2 * np.pi * P["freqs"][k] * P["esc"]["freq"]
    return fq.FrequencyState(w, P["esc"], P["inc"], P["diag"], P["Zs"], P["le"], P["ports"],
                             P["z0"], factor=factor)


def solve_point_lanes(P, fs, Vrest, tol):
    """One frequency point in mixed precision with the ports spread over concurrent
    lanes (one context and host thread each)."""
    lanes = P["lanes"]
    t0 = time.perf_counter()
    lanes.set_frequency(fs.w, fs.DZ, fs.Yle, fs.lu)
    P["host_ms"]["set_frequency"] += (time.perf_counter() - t0) * 1e3
    m, n = P["inc"]["A"].shape
    ns = P["inc"]["Gamma"].shape[1]
    pn = np.asarray(P["ports"]["port_nodes"], dtype=np.int64)
    npt = pn.shape[0]
    z0 = P["z0"]

    def job(c1):
        def run(op):
            tn = op.port_rhs(pn[c1, 0], pn[c1, 1], P["esc"]["Is"])
            return op.solve_mixed(tn, Vrest[:, c1], tol, inner_tol=P["inner_tol"],
                                  inner_maxit=P["settings"]["Inner_Iter"])
        return run
    t0 = time.perf_counter()
    res = lanes.run([job(c1) for c1 in range(npt)])
    P["host_ms"]["solve_mixed"] += (time.perf_counter() - t0) * 1e3
    S = np.zeros((npt, npt), dtype=np.complex128)
    work = []
    for c1, (V, flag, relres, outer, ninner) in enumerate(res):
        work.append({"flag": flag, "relres": relres, "outer": outer, "inner": ninner,
                     "fp64_matvecs": outer + 1, "fp32_matvecs": ninner + outer})
        Vrest[:, c1] = V
    for c1 in range(npt):
        for c2 in range(c1, npt):
            val = 2 * (Vrest[m + ns + pn[c2, 0], c1] - Vrest[m + ns + pn[c2, 1], c1])
            S[c1, c2] = (val - z0) / z0 if c1 == c2 else val / z0
            S[c2, c1] = S[c1, c2]
    return S, work, _point_bytes(P, fs, npt), npt * 2 * (m + ns + n) * 16


def _point_bytes(P, fs, npt, nlanes=1):
    """Host-to-device bytes of one frequency point: each lane's copy of the state (DZ,
    Yle, and the host factors with their permutations when the host factorised), and
    the ports' vectors."""
    from solver_gb300.frequency import export_lu
    m, n = P["inc"]["A"].shape
    N = m + P["inc"]["Gamma"].shape[1] + n
    state = (fs.DZ.nbytes if fs.DZ is not None else 0) + fs.Yle.nnz * 32
    if fs.lu is not None:
        (_, Lc, _), (_, Uc, _), _, _ = export_lu(fs.lu)
        state += (Lc.size + Uc.size) * 24 + (2 * n + 2) * 8 * 2 + 2 * n * 8
    return nlanes * state + npt * (2 * N * 16)


def solve_point(P, fs, Vrest, mode, tol):
    """One frequency point: upload the frequency state, then RHS + solve per port.
    Returns the S-matrix column values and per-port work counts, and H2D/D2H bytes."""
    if mode == "mixed" and P.get("lanes") is not None and len(P["lanes"]) > 1:
        return solve_point_lanes(P, fs, Vrest, tol)
    op = P["op"]
    t0 = time.perf_counter()
    op.set_frequency(fs.w, fs.DZ, fs.Yle, fs.lu)
    P["host_ms"]["set_frequency"] += (time.perf_counter() - t0) * 1e3
    m, n = P["inc"]["A"].shape
    ns = P["inc"]["Gamma"].shape[1]
    pn = np.asarray(P["ports"]["port_nodes"], dtype=np.int64)
    npt = pn.shape[0]
    z0 = P["z0"]
    S = np.zeros((npt, npt), dtype=np.complex128)
    work = []
    for c1 in range(npt):
        t0 = time.perf_counter()
        tn = op.port_rhs(pn[c1, 0], pn[c1, 1], P["esc"]["Is"])
        t1 = time.perf_counter()
        P["host_ms"]["port_rhs"] += (t1 - t0) * 1e3
        if mode == "mixed":
            # warm start from the previous frequency's solution, as the reference does
            V, flag, relres, outer, ninner = op.solve_mixed(tn, Vrest[:, c1], tol,
                                                            inner_tol=P["inner_tol"],
                                                            inner_maxit=P["settings"]["Inner_Iter"])
            P["host_ms"]["solve_mixed"] += (time.perf_counter() - t1) * 1e3
            work.append({"flag": flag, "relres": relres, "outer": outer, "inner": ninner,
                         "fp64_matvecs": outer + 1, "fp32_matvecs": ninner + outer})
        else:
            V, flag, relres, it, rv = op.gmres(tn, Vrest[:, c1], tol, P["settings"]["Inner_Iter"])
            work.append({"flag": flag, "relres": relres, "iter": it,
                         "fp64_matvecs": len(rv) + 1})
        Vrest[:, c1] = V
        for c2 in range(c1, npt):
            val = 2 * (V[m + ns + pn[c2, 0]] - V[m + ns + pn[c2, 1]])
            S[c1, c2] = (val - z0) / z0 if c1 == c2 else val / z0
            S[c2, c1] = S[c1, c2]
    N = m + ns + n
    return S, work, _point_bytes(P, fs, npt), npt * 2 * N * 16


def oracle_port_solves(O, problem, rows, grid, freqs, budget_s, max_solves, tol):
    """Complete port solves of the CPU oracle in the reference's order
    (FFT_solver_QS_S_type.jl:102-208): frequency by frequency, per frequency the SuperLU
    factorisation of SS, then per port its right-hand side (precond_3_3_Kt_fft!) and a
    Householder GMRES solve with its reflectors, warm started from the previous
    frequency's solution of that port. Every operator application runs at the
    reference's 2N extents. Stops after max_solves port solves or once budget_s has
    passed at the end of a solve. Returns the per-solve records and the elapsed time,
    which covers everything from the first factorisation to the last solve."""
    esc, inc, cc, diag, exp, ports, le, Zs, z0, settings = problem
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    A, Gamma = inc["A"], inc["Gamma"]
    m, n = A.shape
    ns = Gamma.shape[1]
    pn = np.asarray(ports["port_nodes"], dtype=np.int64)
    npt = pn.shape[0]
    Vrest = np.zeros((m + ns + n, npt), dtype=np.complex128)
    recs = []
    t0 = time.perf_counter()
    for f in freqs:
        w = 2 * np.pi * f * esc["freq"]
        tf = time.perf_counter()
        fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
        t_lu = time.perf_counter() - tf
        mv = lambda x, fs=fs, w=w: O.ComputeMatrixVectorFTT(
            x, w, inc, FFTCP, FFTCLp, fs["DZ"], fs["Yle"], exp, fs["invZ"], fs["invP"], fs["F"])
        for c1 in range(npt):
            tp = time.perf_counter()
            is_ = np.zeros(n)
            is_[pn[c1, 0]] = esc["Is"]
            is_[pn[c1, 1]] = -esc["Is"]
            tn = O.precond_3_3_Kt_fft(fs["F"], fs["invZ"], fs["invP"], A, Gamma, m, ns, is_)
            V, flag, relres, it, rv = O.gmres_custom(tn, False, tol, int(settings["Inner_Iter"]),
                                                     Vrest[:, c1], mv)
            Vrest[:, c1] = V
            recs.append({"f_hz": float(f), "port": c1, "flag": int(flag), "relres": float(relres),
                         "iters": int(it[1]), "port_s": time.perf_counter() - tp,
                         "lu_s": t_lu if c1 == 0 else 0.0})
            if len(recs) >= max_solves or time.perf_counter() - t0 >= budget_s:
                return recs, time.perf_counter() - t0, npt
    return recs, time.perf_counter() - t0, npt


def cpu_baseline(P):
    """The CPU oracle on the host cores, a bounded sample of the same workload: the
    first frequency's SuperLU factorisation and one complete port solve from a zero
    initial guess (right-hand side, Householder GMRES with reflectors, operator
    applications at the reference's 2N extents with scipy.fft on all cores). A
    frequency point is that factorisation plus one such solve per port."""
    from oracle import peec_oracle as O
    cores = os.cpu_count() or 1
    O.FFT_WORKERS = cores
    (esc, inc, cc, diag, exp, ports, le, li, Zs), freqs, settings, z0, grid = P["oracle"]
    problem = (esc, inc, cc, diag, exp, ports, le, Zs, z0, settings)
    recs, el, npt = oracle_port_solves(O, problem, P["oracle_rows"], grid, freqs[:1], 0.0, 1,
                                       float(settings["tol"]))
    r = recs[0]
    t_point = r["lu_s"] + npt * r["port_s"]
    return {"value": 1.0 / t_point, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"the oracle's SuperLU factorisation at {r['f_hz']:.3g} Hz ({r['lu_s']:.2f} s) "
                       f"and one complete port solve from a zero initial guess ({r['port_s']:.1f} s, "
                       f"{r['iters']} Householder GMRES iterations to {r['relres']:.2e}, operator at "
                       f"the reference 2N extents, scipy.fft x{cores}); a frequency point = the "
                       f"factorisation + {npt} such port solves"),
            "lu_s": r["lu_s"], "port_solve_s": r["port_s"], "gmres_iters": r["iters"]}


def run_small_configs(args):
    """The two small configurations, as one JSON line.
    * crossbar 20x20x4 (two copper bars, one port, 1 GHz, tol 1e-6): the reference
      algorithm (FP64 GMRES) on the GPU, per port solve from a zero initial guess,
      timed over repeated solves, beside the CPU oracle's solve of the same system
      (cpu_baseline leg);
    * the same geometry in mixed precision to 1e-8 at 1 GHz and five log-spaced
      frequencies 100 MHz - 10 GHz: per-frequency port-impedance error against the GPU
      FP64 sweep at 1e-12 (itself parity-tested against the oracle at 1e-10)."""
    from solver_gb300 import api, configs, mesher
    from solver_gb300 import frequency as fq
    from solver_gb300.operator import GpuOperator
    out, freqs, settings, z0, grid = mesher.parse_request(configs.crossbar_20x20x4())
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    op = GpuOperator(inc, exp, diag["P"])
    op.fill(cc["origin"], cc["sx"], cc["sy"], cc["sz"], esc["Lp"], esc["P"])
    w = 2 * np.pi * freqs[0] * esc["freq"]
    st = fq.FrequencyState(w, esc, inc, diag, Zs, le, ports, z0)
    op.set_frequency(w, st.DZ, st.Yle, st.lu)
    n1, n2 = np.asarray(ports["port_nodes"]).reshape(-1, 2)[0]
    tn = op.port_rhs(n1, n2, esc["Is"])
    times = []
    for i in range(args.warmup + 20):
        t = time.perf_counter()
        V, flag, relres, it, rv = op.gmres(tn, None, 1e-6, 100)
        if i >= args.warmup:
            times.append(time.perf_counter() - t)
    gpu_s = float(np.median(times))
    # cpu_baseline leg: the CPU oracle on the same system (reference 2N extents, SuperLU,
    # Householder GMRES)
    from oracle import peec_oracle as O
    fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
    rows = O.fill_rows(cc, esc, *grid)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    mv = lambda x: O.ComputeMatrixVectorFTT(x, w, inc, FFTCP, FFTCLp, fs["DZ"], fs["Yle"], exp,
                                            fs["invZ"], fs["invP"], fs["F"])
    tn_h = np.asarray(tn)
    ct = []
    for i in range(3):
        t = time.perf_counter()
        O.gmres_custom(tn_h, False, 1e-6, 100, np.zeros_like(tn_h), mv)
        ct.append(time.perf_counter() - t)
    cpu_s = float(np.median(ct))
    # mixed precision per frequency against the GPU FP64 sweep
    f3 = [1e9] + list(np.logspace(8, 10, 5))
    nf = len(f3)
    h = api.CirculantSpectra(op)
    exp["gpu_ctx"] = op
    ref = api.FFT_solver_QS_S_type(f3, esc, inc, h, h, diag, ports, z0, le, exp,
                                   {"Inner_Iter": 200, "tol": np.full(nf, 1e-12)}, Zs)
    t = time.perf_counter()
    got = api.FFT_solver_QS_S_type(f3, esc, inc, h, h, diag, ports, z0, le, exp,
                                   {"Inner_Iter": 100, "tol": np.full(nf, 1e-8)}, Zs,
                                   mode="mixed")
    mixed_s = time.perf_counter() - t
    errs = [float(np.max(np.abs(got["Z"][:, :, k] - ref["Z"][:, :, k])) /
                  np.max(np.abs(ref["Z"][:, :, k]))) for k in range(nf)]
    exp.pop("gpu_ctx", None)
    op.close()
    print(json.dumps({
        "metric": "small configurations: crossbar 20x20x4 FP64 plain and mixed per frequency",
        "crossbar_fp64": {"port_solves_per_s": 1.0 / gpu_s, "solve_ms": gpu_s * 1e3,
                          "gmres_iters": int(it[1]), "flag": int(flag), "relres": relres,
                          "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "port solves/s",
                                           "cores": os.cpu_count() or 1, "kind": "port",
                                           "sample": "one oracle GMRES solve of the same system"}},
        "crossbar_mixed": {"freqs_hz": f3, "z_rel_err_vs_fp64_1e-12": dict(
            zip([f"{f:.4g}" for f in f3], errs)), "max_err": max(errs),
            "freq_point_solves_per_s": nf / mixed_s,
            "flags": sorted({int(r["flag"]) for r in got["info"]})}}), flush=True)


def run_reference(args):
    """The reference arm: the CPU oracle restatement of the reference path on the host
    cores (the reference itself is Julia, absent on both machines), built from its own
    mesher restatement and C fill. Each timed step is one complete port solve in the
    reference's frequency x port order, the SuperLU factorisation of a frequency charged
    to its first port. The metric is the completed port solves / ports per elapsed
    second. At most --steps solves run, and no more once the time budget is spent; the
    line reports the solves actually timed. Warm-up steps are one operator application
    each. Rank 0 alone runs; other ranks exit."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import mesher_ref as OM
    from oracle import peec_oracle as O
    from solver_gb300 import configs
    cores = os.cpu_count() or 1
    O.FFT_WORKERS = cores
    req = configs.random_128x128x64() if args.grid is None else configs.random_mixed(tuple(args.grid))
    t = time.perf_counter()
    out, freqs, settings, z0, grid = OM.parse_request(req)
    mesh_s = time.perf_counter() - t
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    t = time.perf_counter()
    rows = O.fill_rows(cc, esc, *grid)
    fill_s = time.perf_counter() - t
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    tol = float(settings["tol"])
    w0 = 2 * np.pi * freqs[0] * esc["freq"]
    fs0 = O.frequency_setup(w0, esc, inc, diag, Zs, le, ports, z0)
    N = inc["A"].shape[0] + inc["A"].shape[1] + inc["Gamma"].shape[1]
    x = np.random.default_rng(0).standard_normal(N) + 0j
    for _ in range(args.warmup):
        O.ComputeMatrixVectorFTT(x, w0, inc, FFTCP, FFTCLp, fs0["DZ"], fs0["Yle"], exp,
                                 fs0["invZ"], fs0["invP"], fs0["F"])
    del fs0
    problem = (esc, inc, cc, diag, exp, ports, le, Zs, z0, settings)
    recs, elapsed, npt = oracle_port_solves(O, problem, rows, grid, freqs, args.ref_budget,
                                            args.steps, tol)
    done = len(recs)
    v = (done / npt) / elapsed
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": done,
            "steps_requested": args.steps, "warmup": args.warmup,
            "ms_per_step": elapsed * 1e3 / done, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "complex128", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD if args.grid is None else f"random {args.grid}",
                       "grid": list(grid), "N": int(N),
                       "step": "one complete port solve (the frequency's SuperLU factorisation "
                               "charged to its first port); value = port solves / ports / s"},
            "timed": {"elapsed_s": elapsed, "port_solves": done, "budget_s": args.ref_budget,
                      "solves": recs, "mesh_s": mesh_s, "fill_s": fill_s,
                      "note": "only the solves listed ran inside the timed region; nothing "
                              "is extrapolated"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": (f"{done} complete oracle port solves in the reference's "
                                        f"frequency x port order from {freqs[0]:.3g} Hz, warm "
                                        f"started, SuperLU per frequency, operator at the "
                                        f"reference 2N extents with scipy.fft x{cores}, mesher "
                                        f"and fill from the oracle")},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line["native_so_loaded"] = loaded_native_libs()
    print(json.dumps(line), flush=True)


def loaded_native_libs():
    """The shared objects of this repository mapped into this process (Linux)."""
    try:
        maps = Path("/proc/self/maps").read_text().splitlines()
    except OSError:
        return None
    root = str(ROOT)
    libs = sorted({ln.split()[-1] for ln in maps
                   if ln.split() and ln.split()[-1].startswith(root) and ".so" in ln})
    return [os.path.relpath(p_, root) for p_ in libs]


def ris_problem(grid=(48, 48, 16), seed=3):
    """A dense RIS workload on a voxel mesh: the mesh's incidence and ports, and its bodies
    as the RIS solver takes them (each edge's Lp brick, each surface's voxel face: vertex
    coordinates, cross-sections / areas, centres), from which the device fills the dense
    Lp blocks and P; R, Cd and the dielectric edges from the mesh's diagonals. Seeded and
    synthetic."""
    from solver_gb300 import configs, mesher, ris
    req = configs.random_mixed(tuple(grid), s=5e-5, p=0.3, seed=seed, nports=4,
                               freqs=[1e8, 1e9, 3e9, 1e10], tol=1e-8)
    out, freqs, settings, z0, g = mesher.parse_request(req)
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    volumi, superfici = ris.voxel_bodies(inc, exp, g, (cc["sx"], cc["sy"], cc["sz"]))
    R = np.real(np.asarray(diag["R"])).sum(axis=1)
    Cd = np.real(np.asarray(diag["Cd"]))
    has = (Cd > 0).any(axis=1)
    Cd_eff = np.zeros(R.size)
    Cd_eff[has] = 1.0 / np.where(Cd[has] > 0, 1.0 / np.where(Cd[has] > 0, Cd[has], 1.0),
                                 0.0).sum(axis=1)
    volumi.update({"R": R, "Cd": Cd_eff,
                   "indici_dielettrici": np.flatnonzero((R == 0) & (Cd_eff > 0)),
                   "Zs_part": np.zeros(R.size)})
    return dict(esc=esc, inc=inc, ports=ports, volumi=volumi, superfici=superfici,
                freqs=list(freqs), grid=list(g))


def ris_fill_cpu(P, k=1500):
    """The oracle's dense fill (oracle/ris_fill.py, C with OpenMP on every host core) on a
    sample: P of the first k surfaces. Returns (pairs per second, sample text)."""
    from oracle import ris_fill
    sup = {"estremi_celle": np.asarray(P["superfici"]["estremi_celle"])[:k],
           "S": np.asarray(P["superfici"]["S"])[:k]}
    empty = {"coordinate": np.zeros((0, 24)), "S": np.zeros(0)}
    ris_fill.dense_fill(empty, {"estremi_celle": sup["estremi_celle"][:50],
                                "S": sup["S"][:50]}, 0, 0, 0)  # build and load
    t = time.perf_counter()
    ris_fill.dense_fill(empty, sup, 0, 0, 0, esc_P=P["esc"]["P"])
    dt = time.perf_counter() - t
    pairs = k * (k + 1) // 2
    return pairs / dt, (f"P of the first {k} surfaces ({pairs} pairs, {dt:.2f} s) with the "
                        f"oracle's C fill on {os.cpu_count() or 1} threads")


def run_ris(args):
    """The dense RIS configuration: the dense Lp blocks and P filled on the device from the
    mesh's bodies (calcola_Lp / calcola_P), the dense operator's FP32 and FP64 applications
    against the HBM roofline, and the RIS frequency x port loop (4 ports x 4 frequencies,
    1e-8) in FP64 and mixed precision with SS factorised on the GPU; beside them the
    oracle's fill (a sample) and its RIS operator and GMRES (one port solve) on the host
    cores. One JSON line."""
    import torch
    from solver_gb300 import ris
    t0 = time.perf_counter()
    P = ris_problem(tuple(args.grid) if args.grid else (48, 48, 16))
    setup_s = time.perf_counter() - t0
    op = ris.DenseOperator.from_geometry(P["inc"], P["volumi"], P["superfici"], P["esc"], 1)
    mx, my, mz = P["inc"]["mx"], P["inc"]["my"], P["inc"]["mz"]
    ns = P["inc"]["Gamma"].shape[1]
    entries = mx * mx + my * my + mz * mz + ns * ns
    # the dense fill (calcola_Lp + calcola_P on the device), timed as a second fill of the
    # operator in place: every pair of the upper triangles, the Lp self terms, P's diagonal
    torch.cuda.synchronize()
    t = time.perf_counter()
    op.fill(P["volumi"], P["superfici"], P["esc"], 1)
    fill_s = time.perf_counter() - t
    pairs = sum(k * (k + 1) // 2 for k in (mx, my, mz, ns))
    fill = {"ms": fill_s * 1e3, "pairs": int(pairs), "pairs_per_s": pairs / fill_s,
            "nonfinite": op.nonfinite, "kernel": "k_ris_pairs (FP64, one thread per pair)"}
    gs = {"Inner_Iter": 300, "tol": [1e-8] * len(P["freqs"])}
    run = lambda mode: ris.iter_solver_QS_S_type(P["freqs"], P["esc"], P["inc"], None, None,
                                                 P["ports"], {}, gs, P["volumi"], False, 1, 50.0,
                                                 mode=mode, op=op, lu="device")
    run("mixed")  # warm-up: graphs, module load
    w = 2 * np.pi * P["freqs"][0] * P["esc"]["freq"]
    st = ris.RisState(w, P["esc"], P["inc"], op.diag_Lp, op.diag_P, P["ports"], {},
                      P["volumi"], False, 50.0)
    op.set_frequency(w, st.DZ, st.Yle, st.lu)
    prof32 = op.profile_matvec(1, 20)
    prof64 = op.profile_matvec(0, 5)
    peak, peak_kind = load_peaks()
    res = {}
    clocks = Clocks(0)
    for mode in ("fp64", "mixed"):
        torch.cuda.synchronize()
        t = time.perf_counter()
        out = run(mode)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        res[mode] = {"port_solves_per_s": len(out["info"]) / dt, "wall_s": dt,
                     "flags": sorted({r["flag"] for r in out["info"]}),
                     "iters_mean": float(np.mean([r["niter"] for r in out["info"]]))}
        res[mode]["S"] = out["S"]
    clk = clocks.stop()
    zerr = float(np.max(np.abs(res["mixed"]["S"] - res["fp64"]["S"])) /
                 np.max(np.abs(res["fp64"]["S"])))
    for mode in res:
        del res[mode]["S"]
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import peec_oracle as O
        from oracle import ris_ref as RO
        Lp_h, P_h = op.dense_data()
        stc = RO.frequency_setup(w, P["esc"], P["inc"], P_h, Lp_h, P["ports"], {},
                                 P["volumi"], False, 50.0)
        mv = lambda x: RO.ComputeMatrixVectorRis(x, w, P["inc"], stc["P"], stc["Lp"],
                                                 stc["Z_self"], stc["Yle"], stc["invZ"],
                                                 stc["invP"], stc["F"])
        pn = np.asarray(P["ports"]["port_nodes"]).reshape(-1, 2)
        isv = np.zeros(op.n)
        isv[pn[0, 0]], isv[pn[0, 1]] = P["esc"]["Is"], -P["esc"]["Is"]
        tn = RO.precond_3_3_Kt_S(stc["F"], stc["invZ"], stc["invP"], P["inc"]["A"],
                                 P["inc"]["Gamma"], op.m, ns, isv)
        t = time.perf_counter()
        _x, fl, _rr, it, rv = O.gmres_custom(tn, False, 1e-8, 300, None, mv)
        dt = time.perf_counter() - t
        cpu = {"value": 1.0 / dt, "unit": "port solves/s", "cores": os.cpu_count() or 1,
               "kind": "port", "sample": f"one FP64 port solve at {P['freqs'][0]:.3g} Hz from "
               f"a zero guess ({len(rv) - 1} GMRES iterations, flag {fl}); the oracle's RIS "
               "operator with numpy/BLAS dense products on every host core"}
        del Lp_h, P_h
        rate, sample = ris_fill_cpu(P)
        fill["cpu_baseline"] = {"value": rate, "unit": "pairs/s", "kind": "port",
                                "cores": os.cpu_count() or 1, "sample": sample}
    ms32, ms64 = prof32["z"], prof64["z"]
    op.close()
    print(json.dumps({
        "metric": "dense RIS solver: port solves/s at 1e-8 (4 ports x 4 frequencies); dense "
                  "fill pairs/s; dense operator GB/s", "value": res["mixed"]["port_solves_per_s"],
        "unit": "port solves/s", "higher_is_better": True, "dtype": "f32 dense products, "
        "float-float refinement residuals over FP64 products", "data": "synthetic",
        "config": {"workload": f"RIS dense fill and solver on random_mixed {P['grid']} (Bernoulli 0.3,"
                   f" seed 3): m = {op.m}, ns = {ns}, n = {op.n}; Lp blocks {mx}/{my}/{mz}, "
                   f"P {ns} x {ns}", "entries": int(entries), "lu": "device",
                   "setup_s": setup_s},
        "fill": fill, "fp64": res["fp64"], "mixed": res["mixed"], "mixed_vs_fp64_S_rel": zerr,
        "dense_products": {"fp32_ms": ms32, "fp64_ms": ms64,
                           "fp32_gbs": 4.0 * entries / (ms32 * 1e-3) / 1e9,
                           "fp64_gbs": 8.0 * entries / (ms64 * 1e-3) / 1e9,
                           "sparse_ms": prof32["sparse"]},
        "roofline": {"bound": "hbm", "kernel": "k_dense_gemv<float> (4 blocks)",
                     "achieved": 4.0 * entries / (ms32 * 1e-3) / 1e9, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": 4.0 * entries / (ms32 * 1e-3) / 1e9 / peak,
                     "bytes_per_application": int(4 * entries)},
        "cpu_baseline": cpu, "clocks": clk}), flush=True)


def run_batched_sweep(args):
    """The batched-sweep configuration: 12 uneven copper grids (32x32x16 .. 96x96x48),
    64 frequencies each, one port, mixed precision to 1e-8, geometries swept concurrently
    (one context and host thread each). Prints one JSON line with the throughput."""
    from solver_gb300 import api, configs
    from solver_gb300.fill_cache import RowCache
    reqs = configs.batched_sweep()
    cache = RowCache() if args.reuse_fills else None
    t = time.perf_counter()
    res = api.sweep_many(reqs, mode="mixed", concurrency=args.lanes, row_cache=cache, lu=args.lu)
    dt = time.perf_counter() - t
    systems = sum(len(r["info"]) for r in res)
    print(json.dumps({"metric": "batched sweep: port solves/s (12 grids x 64 frequencies, 1e-8)",
                      "value": systems / dt, "unit": "port solves/s", "systems": systems,
                      "wall_s": dt, "concurrency": args.lanes, "lu": args.lu,
                      "krylov_loop": args.krylov_loop, "lu_solve": args.lu_solve,
                      "fills": None if cache is None else {"filled": cache.misses,
                                                           "reused": cache.hits},
                      "flags": sorted({r["flag"] for x in res for r in x["info"]}),
                      "max_relres": max(r["relres"] for x in res for r in x["info"]),
                      "inner_iters_mean": float(np.mean([r["niter"] for x in res
                                                          for r in x["info"]]))}),
          flush=True)


def run_adjoint(args):
    """The adjoint-gradient configuration: d|Z|/d sigma_v for every conductor voxel of a
    96x96x32 Bernoulli(0.3) copper grid (seed 5, one port) at 8 frequencies 100 MHz -
    5 GHz, from the mixed-precision solves (reciprocity: no second solve), checked
    against the FP64 solves' gradient and against central finite differences
    (h = 1e-6 sigma, FP64 GMRES to 1e-12) on 16 seeded voxels. One JSON line."""
    from solver_gb300 import configs, gradient as G, mesher
    freqs = np.logspace(np.log10(1e8), np.log10(5e9), 8)
    req = configs.random_copper((96, 96, 32), p=0.3, seed=5, nports=1, freqs=freqs, tol=1e-8)
    P = G.PortImpedanceProblem(mesher.parse_request(req))
    rng = np.random.default_rng(5)
    vox = rng.choice(P.conductor_voxels, size=16, replace=False)
    rows = []
    t_grad = 0.0
    for k in range(len(freqs)):
        t = time.perf_counter()
        absZ, gmx, _ = P.solve(k, mode="mixed")
        t_grad += time.perf_counter() - t
        _, g64, _ = P.solve(k, mode="fp64", maxit=600)
        fd = P.finite_difference(k, vox, h_rel=1e-6) if k in (0, len(freqs) - 1) else None
        scale = float(np.max(np.abs(g64[P.conductor_voxels])))
        # |Z| of this capacitive (terminals not joined) port moves by max_rel_sensitivity
        # * h when one voxel's sigma moves by h * sigma: far below the FP64 solves'
        # rounding floor, so the finite difference is noise; the gradient itself is
        # pinned by the dense-oracle and bar tests
        sens = float(np.max(np.abs(g64 * P.sigma_ref_voxel)) / absZ)
        rows.append({"f_hz": float(freqs[k]), "absZ": absZ,
                     "mixed_vs_fp64": float(np.max(np.abs(gmx - g64)) / scale),
                     "max_rel_sensitivity": sens,
                     "fd_h1e-6_vs_fp64": (float(np.max(np.abs(fd - g64[vox])) / scale)
                                          if fd is not None else None)})
    print(json.dumps({"metric": "adjoint gradient d|Z|/dsigma_v, 96x96x32 copper, 8 frequencies",
                      "conductor_voxels": int(P.conductor_voxels.size),
                      "mixed_solve_plus_gradient_s_per_freq": t_grad / len(freqs),
                      "per_frequency": rows}), flush=True)
    P.close()


def s_matrix(cols, npt):
    S = np.zeros((npt, npt), dtype=np.complex128)
    for c1, col in cols.items():
        for c2, v in col.items():
            S[c1, c2] = S[c2, c1] = v
    return S


def z_of_s(S, z0):
    """s2z_fft (FFT_solver_QS_S_type.jl:265-274): Z = z0 (I - S)^-1 (I + S)."""
    I = np.eye(len(S))
    return z0 * np.linalg.solve(I - S, I + S)


class LaneTimer:
    """Device span of a lane sweep: an event on the first lane's stream that every other
    lane stream waits on, and the last lane's end joined back into the first stream."""

    def __init__(self, lanes, local):
        import torch
        self.torch = torch
        streams = [o.stream() for o in lanes.ops]
        self.ext = [torch.cuda.ExternalStream(h, device=f"cuda:{local}") for h in streams]

    def start(self):
        ev = self.torch.cuda.Event(enable_timing=True)
        ev.record(self.ext[0])
        for xs in self.ext[1:]:
            xs.wait_event(ev)
        self.e0 = ev

    def stop(self):
        for xs in self.ext[1:]:
            ei = self.torch.cuda.Event()
            ei.record(xs)
            self.ext[0].wait_event(ei)
        e1 = self.torch.cuda.Event(enable_timing=True)
        e1.record(self.ext[0])
        e1.synchronize()
        return self.e0.elapsed_time(e1)


def lane_sweep(P, lanes, seq, get_state, Vrest, tol, mode, solve_kw, timer):
    """Every port at every frequency key of seq on the port lanes, warm started along
    the sequence (PortLanes.sweep). Returns the device span (CUDA events, ms), the wall
    time (s), the S columns per position, the work records and the kernel launches."""
    import threading
    m_, n_ = P["inc"]["A"].shape
    ns_ = P["inc"]["Gamma"].shape[1]
    pn = np.asarray(P["ports"]["port_nodes"], dtype=np.int64)
    cols, work = {}, []
    lock = threading.Lock()
    from solver_gb300 import api as _api

    def record(pos, k, c1, V, flag, relres, outer, ninner):
        col = _api._port_column(V, pn, c1, m_, ns_, P["z0"])
        with lock:
            cols.setdefault(pos, {})[c1] = col
            work.append({"pos": pos, "port": c1, "flag": flag, "relres": relres,
                         "outer": outer, "inner": ninner})

    l0 = sum(o.launch_count() for o in lanes.ops)
    t0 = time.perf_counter()
    if timer is not None:
        timer.start()
    lanes.sweep(seq, get_state, lambda k: None, pn, P["esc"]["Is"], Vrest, lambda k: tol,
                solve_kw, record, mode=mode, device_lu=P["device_lu"])
    gpu_ms = timer.stop() if timer is not None else None
    wall = time.perf_counter() - t0
    if gpu_ms is None:
        gpu_ms = wall * 1e3
    launches = sum(o.launch_count() for o in lanes.ops) - l0
    return gpu_ms, wall, cols, work, launches


def z_errors(seq, cols, Zref, npt, z0):
    """Per frequency key: max |Z - Zref| / max |Zref| at the first visit of the key in seq."""
    out = {}
    for pos, k in enumerate(seq):
        if k in out or pos not in cols or k not in Zref:
            continue
        Z = z_of_s(s_matrix(cols[pos], npt), z0)
        out[k] = float(np.max(np.abs(Z - Zref[k])) / np.max(np.abs(Zref[k])))
    return out


def main():
    args = parse()
    if args.impl != "reference":
        from solver_gb300.operator import GpuOperator
        GpuOperator.DEVICE_LOOP = args.krylov_loop == "device"
        GpuOperator.LU_COMPONENT_MAX = 512 if args.lu_solve == "groups" else 0
    if getattr(args, "adjoint", False):
        run_adjoint(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    if args.batched_sweep:
        run_batched_sweep(args)
        return
    if args.ris:
        run_ris(args)
        return
    if args.small_configs:
        run_small_configs(args)
        return
    ws, rank, local = dist_init()
    P = setup_problem(device=local, grid=args.grid)
    P["inner_tol"] = args.inner_tol
    P["device_lu"] = args.lu == "device"
    # with device LU only the first state carries host factors (the pattern and pivot
    # order); every later frequency's SS is assembled and factorised on the GPU
    factor_first = (lambda k: k == 0) if P["device_lu"] else (lambda k: True)
    op = P["op"]
    nf = len(P["freqs"])
    tol = float(P["settings"]["tol"])
    npt = len(P["ports"]["port_nodes"])
    Vrest = np.zeros((op.N, npt), dtype=np.complex128)
    w_of = lambda k: 2 * np.pi * P["freqs"][k] * P["esc"]["freq"]
    # host states (Yle, SuperLU factors) are built by spawned worker processes; the
    # executor is shared by the pools below, so the workers start only once
    from solver_gb300.frequency import FrequencyPool
    static = (P["esc"], P["inc"], P["diag"], P["Zs"], P["le"], P["ports"], P["z0"])
    nworkers = max(2, min(12, (os.cpu_count() or 4) - 4))
    # make_pool(order, key_of): a pool over the keys of `order`, key q building the state
    # of frequency key_of(q), each state kept once built (lanes share it)
    if args.host_states == "processes":
        ex = FrequencyPool.executor(static, nworkers)
        make_pool = lambda order, key_of, factor_of=None: FrequencyPool(
            static, lambda q: w_of(key_of(q)), order, workers=nworkers, lookahead=nworkers,
            keep=True, executor=ex, factor_of=factor_of)
    else:
        # one worker thread, no child processes (for runs under a profiler)
        from solver_gb300.frequency import StatePrefetcher
        ex = None
        nworkers = 1
        make_pool = lambda order, key_of, factor_of=None: StatePrefetcher(
            lambda q: freq_state(P, key_of(q), (factor_of or (lambda _: True))(q)), order,
            keep=True)
    warm_seq = [i % nf for i in range(args.warmup)]
    seq = [i % nf for i in range(args.warmup, args.warmup + args.steps)]
    # cached states for the device-timed passes (inputs prepared before the timed region)
    cache = make_pool([0] + warm_seq + seq, lambda k: k, factor_first)
    state = cache.get

    # -- operator profile and roofline (FP32 and FP64 convolutions) --------------------------
    op.set_frequency(state(0).w, state(0).DZ, state(0).Yle, state(0).lu)
    info = op.conv_info()
    prof32 = op.profile_matvec(1, args.profile_iters)
    prof64 = op.profile_matvec(0, max(3, args.profile_iters // 4))
    profff = op.profile_matvec(2, max(3, args.profile_iters // 4))
    tuning = op.zpass_tuning()
    staged = {"faces": tuning["face"] != "direct", "edges": tuning["edge"] != "direct"}
    b32, b64 = conv_bytes(info, 1, staged), conv_bytes(info, 0)
    peak, peak_kind = load_peaks()
    if args.profile_only:
        # operator applications only (a few hundred launches): the command ncu captures run
        if rank == 0:
            print(json.dumps({"profile_only": True, "grid": list(P["grid"]), "fp32": prof32,
                              "fp64": prof64, "ff": profff, "fp32_bytes_by_pass": b32,
                              "z_tuning": tuning}),
                  flush=True)
        cache.close()
        if ex is not None:
            ex.shutdown()
        op.close()
        return

    from solver_gb300.api import PortLanes
    nlanes = max(1, min(args.lanes, npt))
    lanes = PortLanes(op, nlanes)
    if P["device_lu"]:
        # each lane's factor pattern and pivot order: one host factorisation (frequency 0),
        # made here, outside the timed regions, as the fill is
        from solver_gb300.api import install_state
        for o in lanes.ops:
            install_state(o, state(0), True)
            # the per-edge data from which the device forms each timed point's DZ
            o.set_edge_state(P["diag"], P["Zs"], P["esc"])
    try:
        timer = LaneTimer(lanes, local)
    except Exception:
        timer = None
    mixed_kw = dict(inner_tol=P["inner_tol"], inner_maxit=P["settings"]["Inner_Iter"])
    fp64_kw = dict(maxit=P["settings"]["Inner_Iter"])
    if P["device_lu"]:
        # device-formed states of the mixed sweeps: the host builds Yle only; DZ and the
        # factorisation of SS happen on the GPU (peec_set_frequency_device)
        from solver_gb300.frequency import DeviceFrequencyState
        n_nodes = P["inc"]["A"].shape[1]
        dev_state = lambda k: DeviceFrequencyState(w_of(k), P["esc"], n_nodes, P["le"], P["ports"],
                                                   P["z0"])
        dev_cache = {}
        cached = lambda k, pos: dev_cache[k] if k in dev_cache else dev_cache.setdefault(k, dev_state(k))
    else:
        cached = lambda k, pos: state(k)
    # warm-up: the first points of the sequence, untimed; they also build the warm starts
    if warm_seq:
        lane_sweep(P, lanes, warm_seq, cached, Vrest, tol, "mixed", mixed_kw, None)

    # -- value: device span of the mixed sweep over the timed points (states built) -------
    for k in sorted(set(seq)):
        state(k)
    barrier(ws)
    sync = (lambda: __import__("torch").cuda.synchronize()) if timer is not None else (lambda: None)
    sync()
    clocks = Clocks(local)
    V_e2e = Vrest.copy()  # the e2e pass starts from the same warm starts
    gpu_ms, wall_v, cols_mx, work, launches = lane_sweep(P, lanes, seq, cached, Vrest, tol,
                                                        "mixed", mixed_kw, timer)
    sync()
    # -- e2e: the same points again through the public calls with host buffers; each
    # point's host state (Yle, SuperLU factorisation, exported factors) is built inside the
    # timed region by worker processes that start on it only now, overlapped with the
    # GPU solves of the points before it
    barrier(ws)
    sync()
    t_e0 = time.perf_counter()
    # keyed by position in the timed sequence: a frequency visited twice is built twice
    # (host states by the worker processes; device states by the lane's own thread, Yle only)
    fresh = None if P["device_lu"] else make_pool(list(range(len(seq))), lambda pos: seq[pos])
    waits = [0.0]

    def fresh_state(k, pos):
        th = time.perf_counter()
        st = dev_state(k) if fresh is None else fresh.get(pos, pos=pos)
        waits[0] += time.perf_counter() - th
        return st
    _, wall_e2e, cols_e2e, _, _ = lane_sweep(P, lanes, seq, fresh_state, V_e2e, tol, "mixed",
                                             mixed_kw, None)
    sync()
    wall_e2e = time.perf_counter() - t_e0
    if fresh is not None:
        fresh.close()
    barrier(ws)
    clk = clocks.stop()
    m_, n_ = P["inc"]["A"].shape
    ns_ = P["inc"]["Gamma"].shape[1]
    h2d = sum(_point_bytes(P, cached(k, None) if P["device_lu"] else state(k), npt, nlanes)
              for k in seq)
    d2h = len(seq) * npt * 2 * (m_ + ns_ + n_) * 16
    value, e2e_v, gpu_s, wall_s = whole_job_rates(ws, args.steps, gpu_ms / 1e3, wall_e2e)

    # -- FP64 plain (reference algorithm) and the FP64-residual mixed variant, on the same
    # lanes and the same points; each warm-started from the warm-up points' solutions
    n64 = min(args.fp64_steps, args.steps)
    seq64 = seq[:n64]
    V64 = np.zeros_like(Vrest)
    fp64 = vres = None
    cols64 = colsr = {}
    if n64:
        if warm_seq:
            lane_sweep(P, lanes, warm_seq, cached, V64, tol, "fp64", fp64_kw, None)
        sync()
        ms64, _, cols64, work64, _ = lane_sweep(P, lanes, seq64, cached, V64, tol, "fp64",
                                                fp64_kw, timer)
        fp64 = {"value": n64 / (ms64 / 1e3), "unit": UNIT, "steps": n64, "lanes": nlanes,
                "timing": "CUDA events spanning the lane streams, host states built beforehand "
                          "(as value)",
                "gmres_iters": [w_["inner"] for w_ in sorted(work64, key=lambda r: (r["pos"], r["port"]))]}
        fp64["mixed_over_fp64"] = value / fp64["value"]
        # mixed with FP64 (not float-float) refinement residuals
        for o in lanes.ops:
            o.set_residual_precision(0)
        Vr = np.zeros_like(Vrest)
        if warm_seq:
            lane_sweep(P, lanes, warm_seq, cached, Vr, tol, "mixed", mixed_kw, None)
        sync()
        msr, _, colsr, workr, _ = lane_sweep(P, lanes, seq64, cached, Vr, tol, "mixed",
                                             mixed_kw, timer)
        for o in lanes.ops:
            o.set_residual_precision(2)
        vres = {"value": n64 / (msr / 1e3), "unit": UNIT, "steps": n64, "lanes": nlanes,
                "dtype": "complex64 convolutions in the inner solves; complex128 refinement "
                         "residuals (FP64 convolutions)",
                "outer_mean": float(np.mean([w_["outer"] for w_ in workr])),
                "inner_mean": float(np.mean([w_["inner"] for w_ in workr])),
                "max_relres": float(max(w_["relres"] for w_ in workr))}

    # -- accuracy: every timed arm's port impedances against FP64 GMRES at 1e-12 on the same
    # frequencies (first visit of each in the timed sequence)
    first = []
    for k in seq:
        if k not in first:
            first.append(k)
    Vref = np.zeros_like(Vrest)
    _, _, cols_ref, work_ref, _ = lane_sweep(P, lanes, first, cached, Vref, 1e-12, "fp64",
                                             dict(maxit=400), None)
    Zref = {k: z_of_s(s_matrix(cols_ref[pos], npt), P["z0"]) for pos, k in enumerate(first)}
    fkey = lambda k: f"{P['freqs'][k]:.4g}"
    err_mx = z_errors(seq, cols_mx, Zref, npt, P["z0"])
    err_e2e = z_errors(seq, cols_e2e, Zref, npt, P["z0"])
    err_64 = z_errors(seq64, cols64, Zref, npt, P["z0"])
    err_r = z_errors(seq64, colsr, Zref, npt, P["z0"])
    accuracy = {
        "reference": "FP64 GMRES to relative residual 1e-12 on the GPU (itself parity-tested "
                     "against the oracle at 1e-10; flag 3 marks a solve that stagnated at its "
                     "smallest residual, ref_max_relres), per frequency; max |Z - Z_ref| / "
                     "max |Z_ref|",
        "ref_flags": sorted({w_["flag"] for w_ in work_ref}),
        "ref_max_relres": float(max(w_["relres"] for w_ in work_ref)),
        "mixed": {fkey(k): v for k, v in err_mx.items()},
        "mixed_e2e": {fkey(k): v for k, v in err_e2e.items()},
        "fp64_plain": {fkey(k): v for k, v in err_64.items()},
        "mixed_fp64_residual": {fkey(k): v for k, v in err_r.items()},
        "max": {"mixed": max(err_mx.values()) if err_mx else None,
                "fp64_plain": max(err_64.values()) if err_64 else None,
                "mixed_fp64_residual": max(err_r.values()) if err_r else None},
        "target": 1e-7}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": gpu_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "complex64 convolutions in the inner solves; float-float (48-bit) "
                 "convolutions + complex128 sparse part in the refinement residuals", "data": "synthetic",
        "config": {"workload": WORKLOAD if args.grid is None else f"random {args.grid}",
                   "grid": list(P["grid"]), "N": int(op.N),
                   "m_edges": int(op.m), "ns_surfaces": int(op.ns), "n_nodes": int(op.n),
                   "l2": "inputs larger than L2 (Krylov basis and spectra > 129 MB)",
                   "parallelism": f"replicas x{ws}", "port_lanes": nlanes,
                   "lu": args.lu, "krylov_loop": args.krylov_loop, "lu_solve": args.lu_solve,
                   "timed_points": [fkey(k) for k in seq]},
        "e2e": {"value": e2e_v, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
                "d2h_bytes_per_step": int(d2h / args.steps),
                "host_states": ("built inside the timed region, no state of a timed point "
                                "existing before it: Yle on the host by each lane's thread; "
                                "DZ formed and SS assembled and factorised on the GPU (one "
                                "host factorisation of frequency 0 in the warm-up fixes the "
                                "pattern and pivot order)")
                               if P["device_lu"] else
                               ("built inside the timed region by worker processes started "
                                "on them only then (no state of a timed point exists before "
                                "it); SS factorised by SuperLU on the host at every point"),
                "host_state_wait_ms_per_step": waits[0] / max(1, nlanes) * 1e3 / args.steps,
                "host_state_workers": 0 if P["device_lu"] else nworkers},
        "gpu_launches": int(launches),
        "clocks": clk,
        "fp64_plain": fp64,
        "mixed_fp64_residual": vres,
        "mixed_work": {"outer_mean": float(np.mean([w_["outer"] for w_ in work])),
                       "inner_mean": float(np.mean([w_["inner"] for w_ in work])),
                       "max_relres": float(max(w_["relres"] for w_ in work)),
                       "flags": sorted({w_["flag"] for w_ in work})},
        "accuracy": accuracy,
        "matvec": {"fp32_ms": prof32["total"], "fp64_ms": prof64["total"],
                   "ff_ms": profff["total"], "ff_ms_by_pass": profff,
                   "fp32_conv_gbs": conv_gbs(b32, prof32), "fp64_conv_gbs": conv_gbs(b64, prof64),
                   "fp32_ms_by_pass": prof32, "fp64_ms_by_pass": prof64,
                   "fp32_bytes_by_pass": b32,
                   "fp32_operator_frac": sum(b32.values()) / (prof32["total"] * 1e-3) / 1e9 / peak},
        "reference_model": {
            "bytes_fp32": reference_model_bytes(P["grid"], 8),
            "effective_gbs_fp32": reference_model_bytes(P["grid"], 8) / (prof32["total"] * 1e-3) / 1e9,
            "note": "pruned 3-pass pencil bytes at the reference's 2N extents over the whole "
                    "FP32 operator application (sparse part included in the time)"},
        "roofline": {"bound": "hbm",
                     "kernel": (f"FP32 z passes (forward z FFT, spectral product, inverse z "
                                f"FFT): faces {ZKERNEL['face'][tuning['face']]}, edges "
                                f"{ZKERNEL['edge'][tuning['edge']]}"),
                     "z_tuning": tuning,
                     "achieved": b32["z"] / (prof32["z"] * 1e-3) / 1e9, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": b32["z"] / (prof32["z"] * 1e-3) / 1e9 / peak,
                     "traffic": z_traffic(P["grid"], tuning), "bytes_per_matvec": b32["z"],
                     "launches_per_matvec": 2 if tuning["edge"] == "staged" else 4},
    }
    line["fill"] = fill_report(P, rank == 0 and ws == 1 and not args.no_cpu_baseline)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(P)
    if rank == 0:
        print(json.dumps(line), flush=True)
    cache.close()
    if ex is not None:
        ex.shutdown()
    lanes.close()
    op.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
