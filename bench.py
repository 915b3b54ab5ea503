#!/usr/bin/env python
"""Benchmark of the GB300 FFT-PEEC solver path.

Metric: frequency-point solves per second at 1e-8 relative (left-preconditioned)
residual on the 128x128x64 synthetic voxel geometry (Bernoulli(0.3) occupancy,
copper / dielectric 50/50, 4 ports, 10 frequencies 10 MHz-10 GHz). One step = one
frequency point: the host sparse-LU factorisation of that frequency's Schur
complement, then for each of the 4 ports its right-hand side and a solve warm
started from the previous frequency's solution (FFT_solver_QS_S_type.jl:60-209).

* value: device throughput of the mixed-precision path (FP32 circulant
  convolutions inside FP64 iterative refinement) -- CUDA events on the library's
  stream around the GPU part of each step (frequency upload + 4 port solves), the
  host LU of each frequency prepared beforehand;
* e2e: the same steps end to end through the public API with host buffers, wall
  clock including the host LU, H2D uploads and D2H of each solution;
* fp64_plain: the reference algorithm (FP64 convolutions, Householder GMRES) timed
  on the first frequency points;
* roofline: the z passes of the FP32 convolutions (forward FFT, 3x3 spectral
  product, inverse FFT), algorithmic bytes from the family descriptors, duration from
  CUDA events around the pass;
* cpu_baseline: the CPU oracle restatement (reference 2N extents, scipy FFT on all
  host cores, SuperLU) -- one operator application + one factorisation, scaled by
  the FP64 GMRES matvec count measured in this run.

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
# average FP64 operator applications per port solve of the reference algorithm on this
# workload's warm-started frequency sequence: GMRES takes 12-23 iterations per port (mean
# 17.3 over the 28 port solves of 7 points, measured by the FP64 leg of this script on a
# GB300), plus the initial residual and the final true-residual check. Used only by
# --impl reference, which has no GPU run to count them; the GPU arm counts its own.
REF_MATVECS_PER_PORT = 19.3


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
    ap.add_argument("--lanes", type=int, default=4,
                    help="concurrent port solves (contexts + host threads), at most the ports")
    ap.add_argument("--inner-tol", type=float, default=1e-7,
                    help="floor of the inner FP32 GMRES relative tolerance")
    ap.add_argument("--profile-iters", type=int, default=20)
    ap.add_argument("--grid", type=int, nargs=3, default=None,
                    help="smaller random Cu/dielectric grid (profiling captures only)")
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


def conv_bytes(info, prec):
    """Algorithmic bytes of the convolution passes per operator application: every
    per-family intermediate written once and read once by the next pass, each
    spectrum read once (face families: 3 real + 3 complex spectra on the shared grid;
    edge families: one real spectrum each), lattice maps (int32) once, compact vectors
    (complex128) read once by the gather and written once by the scatter."""
    c = 16 if prec == 0 else 8
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


def z_traffic(grid):
    """DRAM bytes (read + write) of one operator application's FP32 z passes from the
    committed ncu summary of the 128x128x64 workload; None for other grids."""
    if tuple(grid) != (128, 128, 64):
        return None
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                        "z_traffic_random_128x128x64.md")
    try:
        import re
        m = re.search(r"traffic_bytes_per_matvec:\s*(\d+)", open(path).read())
        return int(m.group(1)) if m else None
    except OSError:
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
    out, freqs, settings, z0, grid = mesher.parse_request(req)
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
    the oracle's C fill with OpenMP on every host core (the cpu_baseline leg)."""
    entries = int(sum(np.asarray(r).size for r in P["rows"].values()))
    out = {"entries": entries, "gpu_ms": P["fill_s"] * 1e3,
           "gpu_entries_per_s": entries / P["fill_s"]}
    if with_cpu:
        from oracle import peec_oracle as O
        t = time.perf_counter()
        O.fill_rows(P["cc"], P["esc"], *P["grid"])
        cpu_s = time.perf_counter() - t
        out.update(cpu_ms=cpu_s * 1e3, cpu_entries_per_s=entries / cpu_s,
                   cpu_cores=os.cpu_count() or 1, cpu_kind="port")
    return out


def freq_state(P, k):
    from solver_gb300 import frequency as fq
    w = 2 * np.pi * P["freqs"][k] * P["esc"]["freq"]
    return fq.FrequencyState(w, P["esc"], P["inc"], P["diag"], P["Zs"], P["le"], P["ports"],
                             P["z0"])


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


def _point_bytes(P, fs, npt):
    from solver_gb300.frequency import export_lu
    m, n = P["inc"]["A"].shape
    N = m + P["inc"]["Gamma"].shape[1] + n
    (_, Lc, _), (_, Uc, _), _, _ = export_lu(fs.lu)
    return (fs.DZ.nbytes + (Lc.size + Uc.size) * 24 + (2 * n + 2) * 8 * 2 + 2 * n * 8 +
            fs.Yle.nnz * 32 + npt * (2 * N * 16))


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


def cpu_baseline(P, mv_per_port, sample_note):
    """The CPU oracle on the host cores: one operator application at the reference's
    2N extents (scipy.fft with all cores) and one SuperLU factorisation."""
    from oracle import peec_oracle as O
    cores = os.cpu_count() or 1
    O.FFT_WORKERS = cores
    Nx, Ny, Nz = P["grid"]
    FFTCP, FFTCLp = O.spectra_from_rows(P["rows"], Nx, Ny, Nz)
    w = 2 * np.pi * P["freqs"][0] * P["esc"]["freq"]
    t = time.perf_counter()
    fs = O.frequency_setup(w, P["esc"], P["inc"], P["diag"], P["Zs"], P["le"], P["ports"], P["z0"])
    t_lu = time.perf_counter() - t
    x = np.random.default_rng(0).standard_normal(P["op"].N) + 0j
    t = time.perf_counter()
    O.ComputeMatrixVectorFTT(x, w, P["inc"], FFTCP, FFTCLp, fs["DZ"], fs["Yle"], P["exp"],
                             fs["invZ"], fs["invP"], fs["F"])
    t_mv = time.perf_counter() - t
    npt = len(P["ports"]["port_nodes"])
    t_point = t_lu + npt * mv_per_port * t_mv
    return {"value": 1.0 / t_point, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"one oracle operator application ({t_mv:.2f} s, reference 2N extents, "
                       f"scipy.fft x{cores} threads, 3 SuperLU solves) + one SuperLU factorisation "
                       f"({t_lu:.2f} s); freq point = LU + {npt} ports x {mv_per_port:.1f} matvecs "
                       f"({sample_note})"),
            "matvec_s": t_mv, "lu_s": t_lu}


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
    ws, rank, local = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return
    from oracle import peec_oracle as O
    from solver_gb300 import configs, mesher
    cores = os.cpu_count() or 1
    O.FFT_WORKERS = cores
    req = configs.random_128x128x64()
    out, freqs, settings, z0, grid = mesher.parse_request(req)
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    rows = O.fill_rows(cc, esc, *grid)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    npt = len(ports["port_nodes"])
    x = np.random.default_rng(0).standard_normal(inc["A"].shape[0] + inc["A"].shape[1] +
                                                   inc["Gamma"].shape[1]) + 0j
    times = []
    for i in range(args.warmup + args.steps):
        k = i % len(freqs)
        w = 2 * np.pi * freqs[k] * esc["freq"]
        t = time.perf_counter()
        fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
        t_lu = time.perf_counter() - t
        t = time.perf_counter()
        O.ComputeMatrixVectorFTT(x, w, inc, FFTCP, FFTCLp, fs["DZ"], fs["Yle"], exp, fs["invZ"],
                                 fs["invP"], fs["F"])
        t_mv = time.perf_counter() - t
        if i >= args.warmup:
            times.append(t_lu + npt * REF_MATVECS_PER_PORT * t_mv)
    t_point = float(np.mean(times))
    v = 1.0 / t_point
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_point * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "complex128", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": (f"per step: one SuperLU factorisation + one oracle "
                                        f"operator application (reference 2N extents, scipy.fft x"
                                        f"{cores}), freq point = LU + {npt} ports x "
                                        f"{REF_MATVECS_PER_PORT} matvecs")},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batched_sweep(args):
    """The batched-sweep configuration: 12 uneven copper grids (32x32x16 .. 96x96x48),
    64 frequencies each, one port, mixed precision to 1e-8, geometries swept concurrently
    (one context and host thread each). Prints one JSON line with the throughput."""
    from solver_gb300 import api, configs
    from solver_gb300.fill_cache import RowCache
    reqs = configs.batched_sweep()
    cache = RowCache() if args.reuse_fills else None
    t = time.perf_counter()
    res = api.sweep_many(reqs, mode="mixed", concurrency=args.lanes, row_cache=cache)
    dt = time.perf_counter() - t
    systems = sum(len(r["info"]) for r in res)
    print(json.dumps({"metric": "batched sweep: port solves/s (12 grids x 64 frequencies, 1e-8)",
                      "value": systems / dt, "unit": "port solves/s", "systems": systems,
                      "wall_s": dt, "concurrency": args.lanes,
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


def main():
    args = parse()
    if getattr(args, "adjoint", False):
        run_adjoint(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    if args.batched_sweep:
        run_batched_sweep(args)
        return
    if args.small_configs:
        run_small_configs(args)
        return
    ws, rank, local = dist_init()
    P = setup_problem(device=local, grid=args.grid)
    P["inner_tol"] = args.inner_tol
    P["host_ms"] = {"set_frequency": 0.0, "port_rhs": 0.0, "solve_mixed": 0.0}
    op = P["op"]
    nf = len(P["freqs"])
    tol = float(P["settings"]["tol"])
    Vrest = np.zeros((op.N, len(P["ports"]["port_nodes"])), dtype=np.complex128)
    # host states (Yle, SuperLU factors) of the next frequencies are built by spawned
    # worker processes while the GPU solves the current one
    from solver_gb300.frequency import FrequencyPool
    order = [0] + [i % nf for i in range(args.warmup + args.steps)]
    static = (P["esc"], P["inc"], P["diag"], P["Zs"], P["le"], P["ports"], P["z0"])
    nworkers = max(2, min(12, (os.cpu_count() or 4) - 4))
    if args.host_states == "processes":
        pf = FrequencyPool(static, lambda k: 2 * np.pi * P["freqs"][k] * P["esc"]["freq"],
                           order, workers=nworkers, lookahead=nworkers, keep=True)
    else:
        # one worker thread, no child processes (for runs under a profiler)
        from solver_gb300.frequency import StatePrefetcher
        nworkers = 1
        pf = StatePrefetcher(lambda k: freq_state(P, k), order, keep=True)
    state = pf.get

    # -- operator profile and roofline (FP32 and FP64 convolutions) --------------------------
    op.set_frequency(state(0).w, state(0).DZ, state(0).Yle, state(0).lu)
    info = op.conv_info()
    prof32 = op.profile_matvec(1, args.profile_iters)
    prof64 = op.profile_matvec(0, max(3, args.profile_iters // 4))
    profff = op.profile_matvec(2, max(3, args.profile_iters // 4))
    b32, b64 = conv_bytes(info, 1), conv_bytes(info, 0)
    peak, peak_kind = load_peaks()
    if args.profile_only:
        # operator applications only (a few hundred launches): the command ncu captures run
        if rank == 0:
            print(json.dumps({"profile_only": True, "grid": list(P["grid"]), "fp32": prof32,
                              "fp64": prof64, "ff": profff, "fp32_bytes_by_pass": b32}),
                  flush=True)
        pf.close()
        op.close()
        return

    # -- mixed-precision timed steps ---------------------------------------------------------
    from solver_gb300.api import PortLanes
    nlanes = max(1, min(args.lanes, len(P["ports"]["port_nodes"])))
    P["lanes"] = PortLanes(op, nlanes)
    lane_streams = [op.stream()] + [o.stream() for o in P["lanes"].ops[1:]]
    try:
        import torch
        ext = torch.cuda.ExternalStream(op.stream(), device=f"cuda:{local}")
        lane_ext = [ext] + [torch.cuda.ExternalStream(h, device=f"cuda:{local}")
                            for h in lane_streams[1:]]
        ev = lambda: torch.cuda.Event(enable_timing=True)
        have_torch = True
    except Exception:
        have_torch = False
    S_mixed = {}
    for i in range(args.warmup):
        k = i % nf
        S_mixed[k], _, _, _ = solve_point(P, state(k), Vrest, "mixed", tol)
    # the timed points: every lane runs its ports through the whole timed frequency
    # sequence on its own (PortLanes.sweep), so one lane's frequency-state upload overlaps
    # the other lanes' solves; the device span runs from an event all lane streams wait
    # on to the last lane's end
    from solver_gb300 import api as _api
    import threading
    seq = [i % nf for i in range(args.warmup, args.warmup + args.steps)]
    m_, n_ = P["inc"]["A"].shape
    ns_ = P["inc"]["Gamma"].shape[1]
    pn = np.asarray(P["ports"]["port_nodes"], dtype=np.int64)
    npt = pn.shape[0]
    cols = {}
    work = []
    rlock = threading.Lock()
    wait_s = [0.0]

    def record(pos, k, c1, V, flag, relres, outer, ninner):
        col = _api._port_column(V, pn, c1, m_, ns_, P["z0"])
        with rlock:
            cols.setdefault(pos, {})[c1] = col
            work.append({"flag": flag, "relres": relres, "outer": outer, "inner": ninner,
                         "fp64_matvecs": outer + 1, "fp32_matvecs": ninner + outer})

    def get_state(k, pos):
        th = time.perf_counter()
        st = pf.get(k, pos=1 + args.warmup + pos)
        with rlock:
            wait_s[0] += time.perf_counter() - th
        return st

    l0 = sum(o.launch_count() for o in P["lanes"].ops)
    barrier(ws)
    if have_torch:
        torch.cuda.synchronize()
    clocks = Clocks(local)
    t_wall0 = time.perf_counter()
    if have_torch:
        e0, e1 = ev(), ev()
        e0.record(ext)
        for xs in lane_ext[1:]:
            xs.wait_event(e0)
    P["lanes"].sweep(seq, get_state, lambda k: None, pn, P["esc"]["Is"], Vrest,
                     lambda k: tol, dict(inner_tol=P["inner_tol"],
                                         inner_maxit=P["settings"]["Inner_Iter"]), record)
    if have_torch:
        for xs in lane_ext[1:]:
            ei = ev()
            ei.record(xs)
            ext.wait_event(ei)
        e1.record(ext)
        e1.synchronize()
        gpu_ms = e0.elapsed_time(e1)
        torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    if not have_torch:
        gpu_ms = t_wall * 1e3
    host_wait = wait_s[0] / max(1, nlanes)
    h2d = d2h = 0
    for pos, k in enumerate(seq):
        Sk = np.zeros((npt, npt), dtype=np.complex128)
        for c1, col in cols[pos].items():
            for c2, v in col.items():
                Sk[c1, c2] = Sk[c2, c1] = v
        S_mixed[k] = Sk
        h2d += _point_bytes(P, state(k), npt)
        d2h += npt * 2 * (m_ + ns_ + n_) * 16
    barrier(ws)
    clk = clocks.stop()
    launches = sum(o.launch_count() for o in P["lanes"].ops) - l0
    value, e2e_v, gpu_s, wall_s = whole_job_rates(ws, args.steps, gpu_ms / 1e3, t_wall)

    # -- FP64 plain (reference algorithm) on the same frequency sequence ---------------------
    # the warm-up points build the same warm starts untimed; then the first fp64_steps of
    # the timed mixed points are timed
    V64 = np.zeros_like(Vrest)
    fp64_ms = 0.0
    work64 = []
    S64 = {}
    n64 = min(args.fp64_steps, args.steps)
    if n64:
        for i in range(args.warmup):
            solve_point(P, state(i % nf), V64, "fp64", tol)
        for i in range(args.warmup, args.warmup + n64):
            k = i % nf
            fs = state(k)
            t0 = time.perf_counter()
            S64[k], w64, _, _ = solve_point(P, fs, V64, "fp64", tol)
            fp64_ms += (time.perf_counter() - t0) * 1e3
            work64 += w64
    fp64_v = n64 / (fp64_ms / 1e3) if n64 else None
    # mixed vs FP64 port quantities (S) at the frequencies both ran
    errs = []
    for k in S64:
        if k in S_mixed:
            a, b = S_mixed[k], S64[k]
            Za = 50 * np.linalg.solve(np.eye(len(a)) - a, np.eye(len(a)) + a)
            Zb = 50 * np.linalg.solve(np.eye(len(b)) - b, np.eye(len(b)) + b)
            errs.append(float(np.max(np.abs(Za - Zb)) / np.max(np.abs(Zb))))
    mv_per_port = float(np.mean([w_["fp64_matvecs"] for w_ in work64])) if work64 else \
        float(REF_MATVECS_PER_PORT)

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
                   "parallelism": f"replicas x{ws}", "port_lanes": nlanes},
        "e2e": {"value": e2e_v, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
                "d2h_bytes_per_step": int(d2h / args.steps),
                "host_state_wait_ms_per_step": host_wait * 1e3 / args.steps,
                "host_state_workers": nworkers},
        "gpu_launches": int(launches),
        "clocks": clk,
        "fp64_plain": {"value": fp64_v, "unit": UNIT, "steps": n64,
                       "mixed_over_fp64": (value / fp64_v) if fp64_v else None,
                       "gmres_iters": [w_["iter"][1] for w_ in work64]},
        "mixed_work": {"outer_mean": float(np.mean([w_["outer"] for w_ in work])),
                       "inner_mean": float(np.mean([w_["inner"] for w_ in work])),
                       "max_relres": float(max(w_["relres"] for w_ in work)),
                       "z_rel_err_vs_fp64": max(errs) if errs else None},
        "matvec": {"fp32_ms": prof32["total"], "fp64_ms": prof64["total"],
                   "ff_ms": profff["total"], "ff_ms_by_pass": profff,
                   "fp32_conv_gbs": conv_gbs(b32, prof32), "fp64_conv_gbs": conv_gbs(b64, prof64),
                   "fp32_ms_by_pass": prof32, "fp64_ms_by_pass": prof64,
                   "fp32_bytes_by_pass": b32},
        "reference_model": {
            "bytes_fp32": reference_model_bytes(P["grid"], 8),
            "effective_gbs_fp32": reference_model_bytes(P["grid"], 8) / (prof32["total"] * 1e-3) / 1e9,
            "note": "pruned 3-pass pencil bytes at the reference's 2N extents over the whole "
                    "FP32 operator application (sparse part included in the time)"},
        "roofline": {"bound": "hbm", "kernel": "k_zconv3<float> + k_zconv1<float> (z passes: "
                     "FFT, spectral product, inverse FFT)",
                     "achieved": b32["z"] / (prof32["z"] * 1e-3) / 1e9, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": b32["z"] / (prof32["z"] * 1e-3) / 1e9 / peak,
                     "traffic": z_traffic(P["grid"]), "bytes_per_matvec": b32["z"],
                     "launches_per_matvec": 4},
    }
    line["fill"] = fill_report(P, rank == 0 and ws == 1 and not args.no_cpu_baseline)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(P, mv_per_port,
                                            "matvec count measured by the FP64 run above")
    if rank == 0:
        print(json.dumps(line), flush=True)
    pf.close()
    P["lanes"].close()
    op.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
