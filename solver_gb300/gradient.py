"""Gradient of a port's impedance magnitude with respect to per-voxel conductivity.

Adjoint by reciprocity. The unpreconditioned PEEC system (the operator of
compute_Matrix_vector_fft.jl:29-77 before its preconditioner)

    K = [[jw Lp + diag(DZ), 0,        A  ],
         [0,                P,       -G' ],
         [-A',              jw G,    Yle ]]

has symmetric circulant blocks (Lp = Lp', P = P') and a symmetric termination block
(Yle), so K' = D1 K D2 with D1 = diag(I, jw I, -I) and D2 = diag(I, I/(jw), -I).
The port voltage val = 2 (phi[n1] - phi[n2]) = c' x, with x = K^-1 b and
b = [0; 0; +Is at n1, -Is at n2], so c = (2/Is) b. The adjoint solve
K' lambda = c is therefore a forward solve: lambda = D2^-1 K^-1 D1^-1 c, whose edge
block is -(2/Is) I (the port's own edge currents). The operator depends on the
conductivity only through DZ, so

    d val / d sigma_v = -lambda' (dK/dsigma_v) x = (2/Is) sum_e (dDZ_e/dsigma_v) I_e^2,

and no second Krylov solve (and no stored Krylov basis) is needed: the gradient reuses
the forward GMRES solution of the frequency sweep.

DZ_e (FFT_solver_QS_S_type.jl:105-116) is the edge's four half resistances (or their
RC parallels, compute_Z_self.jl) plus the surface impedance, keeping the larger real
part for surface edges. A half resistance R = (l/2)/(sigma a b) lies in one voxel
(columns 0 and 2 of the R / Cd / Zsw tables in the edge's first voxel, 1 and 3 in its
second); dR/dsigma = -R/sigma, and the surface-impedance contributions scale as
sigma^(-1/2). The port impedance of a single port is Z = z0 val / (2 z0 - val)
(s2z_fft, FFT_solver_QS_S_type.jl:265-274).
"""
from __future__ import annotations

import math

import numpy as np

from .frequency import z_self


def edge_voxels(incidence_selection, expansions):
    """(v1, v2): 0-based voxel number of the first and second voxel of every edge (an
    x edge at lattice cell (x, y, z) joins voxels (x, y, z) and (x+1, y, z))."""
    Nx, Ny, Nz = expansions["grid"]
    vm = np.asarray(expansions["vox_map"]).ravel()
    cell = np.asarray(expansions["edge_cell"], dtype=np.int64)
    mx, my, mz = (int(incidence_selection[k]) for k in ("mx", "my", "mz"))
    v1 = np.empty(cell.size, dtype=np.int64)
    v2 = np.empty(cell.size, dtype=np.int64)
    offs = (0, mx, mx + my, mx + my + mz)
    lat = ((Nx - 1, Ny, Nz), (Nx, Ny - 1, Nz), (Nx, Ny, Nz - 1))
    step = ((1, 0, 0), (0, 1, 0), (0, 0, 1))
    for c in range(3):
        lc = cell[offs[c]:offs[c + 1]]
        lx, ly, _ = lat[c]
        x = lc % lx
        y = (lc // lx) % ly
        z = lc // (lx * ly)
        a = (z * Ny + y) * Nx + x
        b = ((z + step[c][2]) * Ny + (y + step[c][1])) * Nx + (x + step[c][0])
        v1[offs[c]:offs[c + 1]] = vm[a] - 1
        v2[offs[c]:offs[c + 1]] = vm[b] - 1
    return v1, v2


def edge_sigma(Zs_info, materials_sigma):
    """Conductivity of every edge (both voxels of an edge share its material)."""
    mats = np.asarray(Zs_info["materials"], dtype=np.int64)
    sig = np.asarray(materials_sigma, dtype=np.float64)
    return np.where(mats > 0, sig[np.maximum(mats - 1, 0)], 0.0)


def _par(a, b):
    out = a + b
    both = (a != 0) & (b != 0)
    out[both] = a[both] * b[both] / (a[both] + b[both])
    return out


def dz_edges(w, escalings, diagonals, Zs_info, sigma_voxel, v1, v2, sigma_ref):
    """DZ of every edge for per-voxel conductivities sigma_voxel, and its derivatives
    with respect to the conductivity of the edge's first and second voxel.

    The tables in diagonals / Zs_info were built with the material conductivities
    sigma_ref (per edge); a half resistance scales as sigma_ref/sigma_v, a surface
    impedance contribution as sqrt(sigma_ref/sigma_v)."""
    R = np.asarray(diagonals["R"], dtype=np.float64).copy()
    Cd = np.asarray(diagonals["Cd"]).copy()
    Zsw = np.asarray(Zs_info["Zsw"], dtype=np.complex128).copy()
    cond = sigma_ref > 0
    s1 = np.where(cond, sigma_voxel[np.maximum(v1, 0)], 1.0)
    s2 = np.where(cond, sigma_voxel[np.maximum(v2, 0)], 1.0)
    f1 = np.where(cond, sigma_ref / s1, 1.0)
    f2 = np.where(cond, sigma_ref / s2, 1.0)
    for col, f in ((0, f1), (2, f1), (1, f2), (3, f2)):
        R[:, col] *= f
    for col, f in ((0, f1), (1, f1), (2, f2), (3, f2)):
        Zsw[:, col] *= np.sqrt(f)
    # self impedance and its derivative: z = R (Cd = 0) or 1/(1/R + jwCd)
    Zself = z_self(R, Cd, w)
    dz1 = np.zeros(R.shape[0], dtype=np.complex128)
    dz2 = np.zeros(R.shape[0], dtype=np.complex128)
    for col, s, d in ((0, s1, dz1), (2, s1, dz1), (1, s2, dz2), (3, s2, dz2)):
        r, cd = R[:, col], Cd[:, col]
        rc = (r != 0) & (cd != 0)
        ro = (r != 0) & (cd == 0)
        dzdr = np.zeros_like(dz1)
        dzdr[ro] = 1.0
        zrc = 1.0 / (1.0 / r[rc] + 1j * w * cd[rc])
        dzdr[rc] = zrc ** 2 / r[rc] ** 2
        d += np.where(cond, dzdr * (-r / s), 0.0)
    # surface impedance and its derivative (homogeneous of degree -1/2 in sigma per voxel)
    scale = escalings["R"] * math.sqrt(w / escalings["freq"])
    p1 = _par(Zsw[:, 0], Zsw[:, 1])
    p2 = _par(Zsw[:, 2], Zsw[:, 3])
    Zs = scale * (p1 + p2)
    dzs1 = np.where(cond, -scale * p1 / (2 * s1), 0.0)
    dzs2 = np.where(cond, -scale * p2 / (2 * s2), 0.0)
    # keep the larger real part on surface edges (FFT_solver_QS_S_type.jl:108-115)
    se = np.asarray(Zs_info["surface_edges"], dtype=np.int64)
    zs_wins = np.zeros(R.shape[0], dtype=bool)
    zs_wins[se] = Zs[se].real - Zself[se].real > 0
    self_loses = zs_wins
    Zself_eff = np.where(self_loses, 1j * Zself.imag, Zself)
    Zs_eff = np.where(zs_wins, Zs, 1j * Zs.imag)
    DZ = Zself_eff + Zs_eff.real + 1j * w * np.asarray(diagonals["Lp"]).ravel()
    d1 = np.where(self_loses, 1j * dz1.imag, dz1) + np.where(zs_wins, dzs1.real, 0.0)
    d2 = np.where(self_loses, 1j * dz2.imag, dz2) + np.where(zs_wins, dzs2.real, 0.0)
    return DZ, d1, d2


def port_impedance_and_gradient(V, m, ns, port_nodes, z0, Is, d1, d2, v1, v2, nvox, op=None):
    """|Z| of a one-port geometry and d|Z|/d sigma_v for every voxel from the forward
    solution V = [I; Q; phi] (edge currents first) and the DZ derivatives. With op (a
    GpuOperator) the per-voxel scatter runs on the GPU (peec_adjoint); without, on the
    host."""
    n1, n2 = (int(t) for t in port_nodes)
    val = 2.0 * (V[m + ns + n1] - V[m + ns + n2])
    Z = z0 * val / (2.0 * z0 - val)
    dZ_dval = 2.0 * z0 * z0 / (2.0 * z0 - val) ** 2
    if op is not None:
        g = op.adjoint(V, v1, v2, d1, d2, Is, nvox)
    else:
        I2 = V[:m] ** 2
        g = np.zeros(nvox, dtype=np.complex128)
        ok1, ok2 = v1 >= 0, v2 >= 0
        np.add.at(g, v1[ok1], (2.0 / Is) * d1[ok1] * I2[ok1])
        np.add.at(g, v2[ok2], (2.0 / Is) * d2[ok2] * I2[ok2])
    dZ = dZ_dval * g
    return abs(Z), np.real(np.conj(Z) * dZ) / abs(Z), Z


class PortImpedanceProblem:
    """A one-port geometry on the GPU with per-voxel conductivities: forward solves of the
    port (FP64 GMRES as in the reference, or the mixed solve), |Z| and its gradient over
    the voxels (reciprocity, see the module docstring), and central finite differences.

    parsed: mesher.parse_request output (out, freqs, settings, z0, grid)."""

    def __init__(self, parsed, op=None, device=0):
        from .operator import GpuOperator
        out, freqs, settings, z0, grid = parsed
        (self.esc, self.inc, self.cc, self.diag, self.exp, self.ports, self.le, _li,
         self.Zs) = out
        self.freqs = np.asarray(freqs, dtype=np.float64)
        self.z0 = z0
        self.settings = settings
        if len(np.asarray(self.ports["port_nodes"]).reshape(-1, 2)) != 1:
            raise ValueError("the impedance gradient is defined for one-port geometries")
        self.m, self.n = self.inc["A"].shape
        self.ns = self.inc["Gamma"].shape[1]
        self.v1, self.v2 = edge_voxels(self.inc, self.exp)
        self.nvox = int(np.max(self.exp["vox_map"]))
        self.sigma_edge = edge_sigma(self.Zs, self._material_sigma())
        self.sigma_ref_voxel = np.zeros(self.nvox)
        cond = self.sigma_edge > 0
        self.sigma_ref_voxel[self.v1[cond]] = self.sigma_edge[cond]
        self.sigma_ref_voxel[self.v2[cond]] = self.sigma_edge[cond]
        self.conductor_voxels = np.flatnonzero(self.sigma_ref_voxel > 0)
        self._own = op is None
        if op is None:
            op = GpuOperator(self.inc, self.exp, self.diag["P"], device=device)
            op.fill(self.cc["origin"], self.cc["sx"], self.cc["sy"], self.cc["sz"],
                    self.esc["Lp"], self.esc["P"])
        self.op = op
        self._x = {}

    def _material_sigma(self):
        mats = np.asarray(self.Zs["materials"], dtype=np.int64)
        # per material: the conductivity the diagonals were built with (copper tables
        # carry R != 0 exactly where sigma != 0); recovered from the R table itself
        R = np.asarray(self.diag["R"], dtype=np.float64)
        out = np.zeros(int(mats.max()) if mats.size else 0)
        return out if out.size == 0 else self._sigma_from_R(R, mats, out)

    def _sigma_from_R(self, R, mats, out):
        # R_half = (l/2) / (sigma a b) * escal_R  ->  sigma = (l/2) / (R_half a b) * escal_R
        sx, sy, sz = self.cc["sx"], self.cc["sy"], self.cc["sz"]
        s_of = [(sx, sy, sz), (sy, sx, sz), (sz, sy, sx)]
        mx, my, mz = (int(self.inc[k]) for k in ("mx", "my", "mz"))
        offs = (0, mx, mx + my, mx + my + mz)
        for c in range(3):
            l_, a_, b_ = s_of[c]
            for e in range(offs[c], offs[c + 1]):
                k = mats[e]
                if k > 0 and out[k - 1] == 0 and R[e, 0] > 0:
                    out[k - 1] = 0.5 * l_ / (R[e, 0] / self.esc["R"] * a_ * b_)
        return out

    def close(self):
        if self._own and self.op is not None:
            self.op.close()
        self.op = None

    def _state(self, w, sigma_voxel):
        from .frequency import FrequencyState
        DZ, d1, d2 = dz_edges(w, self.esc, self.diag, self.Zs, sigma_voxel, self.v1, self.v2,
                              self.sigma_edge)
        fs = FrequencyState(w, self.esc, self.inc, self.diag, self.Zs, self.le, self.ports,
                            self.z0, DZ=DZ)
        return fs, d1, d2

    def solve(self, k, sigma_voxel=None, mode="fp64", tol=None, warm=True, maxit=None):
        """|Z|, d|Z|/d sigma over all voxels and Z at frequency index k."""
        sv = self.sigma_ref_voxel if sigma_voxel is None else np.asarray(sigma_voxel, float)
        w = 2 * np.pi * self.freqs[k] * self.esc["freq"]
        fs, d1, d2 = self._state(w, sv)
        self.op.set_frequency(fs.w, fs.DZ, fs.Yle, fs.lu)
        n1, n2 = np.asarray(self.ports["port_nodes"]).reshape(-1, 2)[0]
        tn = self.op.port_rhs(n1, n2, self.esc["Is"])
        tol = float(self.settings["tol"]) if tol is None else tol
        maxit = int(self.settings["Inner_Iter"]) if maxit is None else int(maxit)
        x0 = self._x.get(mode) if warm else None
        if mode == "fp64":
            V, flag, relres, it, rv = self.op.gmres(tn, x0, tol, maxit)
        else:
            V, flag, relres, outer, inner = self.op.solve_mixed(tn, x0, tol, inner_maxit=maxit)
        # flag 3: GMRES stagnated at the rounding floor of the system (relres is then the
        # best this arithmetic reaches); anything else that did not converge is an error
        if flag != 0 and not (flag == 3 and relres <= max(1e2 * tol, 1e-8)):
            raise RuntimeError(f"port solve did not converge (flag {flag}, relres {relres})")
        self._x[mode] = V
        absZ, g, Z = port_impedance_and_gradient(V, self.m, self.ns, (n1, n2), self.z0,
                                                 self.esc["Is"], d1, d2, self.v1, self.v2,
                                                 self.nvox, op=self.op)
        return absZ, g, Z

    def finite_difference(self, k, voxels, h_rel=1e-6, tol=1e-12, maxit=600):
        """Central differences of |Z| in the conductivity of each voxel (FP64 solves to
        tol, or to GMRES's rounding floor where that is higher: the difference then
        carries that floor divided by h_rel)."""
        out = []
        for v in voxels:
            h = h_rel * self.sigma_ref_voxel[v]
            vals = []
            for sgn in (1.0, -1.0):
                sv = self.sigma_ref_voxel.copy()
                sv[v] += sgn * h
                vals.append(self.solve(k, sv, mode="fp64", tol=tol, warm=False, maxit=maxit)[0])
            out.append((vals[0] - vals[1]) / (2 * h))
        return np.asarray(out)

    def directional_difference(self, k, direction, h=1e-4, tol=1e-12, maxit=600):
        """Central difference of |Z| along sigma + t * direction (t = +-h) with FP64
        solves: the derivative d|Z|/dt, to be compared with gradient . direction. A
        direction over many voxels (e.g. sigma_v * sign(g_v)) moves |Z| far more than one
        voxel does, so the difference stays well above the solves' rounding floor."""
        d = np.asarray(direction, dtype=np.float64)
        vals = []
        for sgn in (1.0, -1.0):
            sv = self.sigma_ref_voxel + sgn * h * d
            vals.append(self.solve(k, sv, mode="fp64", tol=tol, warm=False, maxit=maxit)[0])
        return (vals[0] - vals[1]) / (2 * h)


def impedance_magnitude_function():
    """torch.autograd.Function for |Z_port|(sigma): forward runs the port solve at the
    given per-voxel conductivities (a torch tensor), backward returns the reciprocity
    gradient. apply(sigma, problem, k, mode)."""
    import torch

    class ImpedanceMagnitude(torch.autograd.Function):
        @staticmethod
        def forward(ctx, sigma, problem, k, mode="mixed"):
            absZ, g, _ = problem.solve(k, sigma.detach().cpu().numpy(), mode=mode)
            ctx.save_for_backward(torch.as_tensor(g, dtype=sigma.dtype))
            return torch.tensor(absZ, dtype=sigma.dtype)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            return grad_out * g, None, None, None

    return ImpedanceMagnitude
