"""Shape and incidence sensitivities of airfoil force coefficients.

The gradient is the discrete adjoint of the FP64 device residual (include/aero_adjoint.h):
the primal is converged on the deformed mesh, (dR/dU)^T lam = -dJ/dU is solved with the
primal's pseudo-time smoother (or GMRES preconditioned by it), and

    dJ/d(alpha) = dJ/d(alpha)|_U + lam^T dR/d(alpha)          (far-field state)
    dJ/d(a_k)   = dJ/dX . m_k   + lam^T (dR/dX . m_k)          (m_k: Hicks-Henne mode k)

with the geometry tangents of each mode from aero_mesh_geometry_tangent, or with dJ/dX for
every node from one reverse pass (aero_adjoint_node_vjp) contracted with the modes. AirfoilForces is
the torch.autograd.Function over (amplitudes, alpha) -> (CD, CL). There is no reference
counterpart: AeroCFD has no shape parameterisation and no adjoint.
"""

from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import Solver, capi, deform, geometry_tangent, hicks_henne_modes


def converged_case(case: capi.CaseDesc, alpha_deg: float, precision: int, max_iters: int,
                   rho_target: float) -> capi.CaseDesc:
    """The case at incidence alpha_deg, stopping only on the density-residual ratio."""
    c = capi.CaseDesc()
    C.pointer(c)[0] = case
    c.aoa_deg = float(alpha_deg)
    c.precision = int(precision)
    c.iterations = int(max_iters)
    c.residual_reduction_target = 0.0  # the reference's ratio rule never fires
    c.density_l2_target = float(rho_target)
    return c


@dataclass
class PrimalResult:
    solver: Solver
    mesh: capi.Mesh
    cd: float
    cl: float
    iterations: int
    rho_ratio: float
    seconds: float


@dataclass
class ShapeProblem:
    """Airfoil force coefficients as functions of Hicks-Henne amplitudes and incidence.

    mesh: a generated O-grid (ogrid_synthetic / ogrid_reference); case: its flow case;
    peaks / upper: bump positions in (0, 1) and sides; width: the bump exponent.
    """

    mesh: capi.Mesh
    case: capi.CaseDesc
    peaks: np.ndarray
    upper: np.ndarray
    width: float = 3.0
    max_iters: int = 200000
    rho_target: float = 1e-12
    chunk: int = 5000
    adjoint_max_iters: int = 400000
    adjoint_tol: float = 1e-10
    adjoint_cfl: float | None = None
    # "smoother": the primal's RK3 pseudo-time iteration, which converges at the primal's rate
    # wherever the primal converged; "krylov": GMRES preconditioned by smoother sweeps
    # (adjoint_max_iters then counts Arnoldi steps)
    adjoint_method: str = "smoother"
    krylov_restart: int = 40
    krylov_smooth: int = 10
    primal_precision: int = capi.PRECISION_FP64
    # "tangent": lam^T dR/dX . m_k from one forward geometry tangent per mode; "reverse":
    # dJ/dX for every node in one reverse pass, then dJ/da_k = dJ/dX . m_k (any number of modes
    # at the cost of one)
    geometry_product: str = "tangent"
    modes: np.ndarray = field(init=False)
    last_adjoint_seconds: float = field(init=False, default=0.0)
    last_adjoint_iterations: int = field(init=False, default=0)
    last_adjoint_ratio: float = field(init=False, default=0.0)

    def __post_init__(self):
        self.peaks = np.asarray(self.peaks, np.float64)
        self.upper = np.asarray(self.upper, np.int32)
        self.modes = hicks_henne_modes(self.mesh, self.peaks, self.upper, self.width)

    def mesh_at(self, amplitudes) -> capi.Mesh:
        a = np.asarray(amplitudes, np.float64)
        pts = self.mesh.points.reshape(-1, 3) + np.tensordot(a, self.modes, axes=1)
        return deform(self.mesh, pts)

    def solve(self, amplitudes, alpha_deg: float, precision: int | None = None) -> PrimalResult:
        """Converge the primal on the deformed mesh (density-residual ratio rho_target)."""
        prec = self.primal_precision if precision is None else precision
        mesh = self.mesh_at(amplitudes)
        case = converged_case(self.case, alpha_deg, prec, self.max_iters, self.rho_target)
        s = Solver(mesh, case)
        t0 = time.perf_counter()
        done, last = 0, None
        while done < self.max_iters:
            _, recs = s.run(min(self.chunk, self.max_iters - done))
            if recs.size == 0:
                break
            done += recs.size
            last = recs[-1]
            if last["flags"] & capi.REC_CONVERGED:
                break
        secs = time.perf_counter() - t0
        if last is None:
            raise RuntimeError("primal ran no iterations")
        return PrimalResult(s, mesh, float(last["cd"]), float(last["cl"]), done, float(last["residual_rho_ratio"]),
                            secs)

    def adjoint_solver(self, primal: PrimalResult) -> Solver:
        """The FP64 context the adjoint runs in: the primal's own, or an FP64 copy of an FP32
        primal's state."""
        if primal.solver.case.precision == capi.PRECISION_FP64:
            return primal.solver
        case = capi.CaseDesc()
        C.pointer(case)[0] = primal.solver.case
        case.precision = capi.PRECISION_FP64
        s = Solver(primal.mesh, case)
        s.set_state(primal.solver.get_state())
        return s

    def gradient(self, primal: PrimalResult, w_cd: float, w_cl: float):
        """(dJ/da [n], dJ/d(alpha) per degree) for J = w_cd CD + w_cl CL at the primal's state."""
        s = self.adjoint_solver(primal)
        cfl = self.adjoint_cfl if self.adjoint_cfl is not None else float(self.case.cfl_max)
        t0 = time.perf_counter()
        s.adjoint_linearize(w_cd, w_cl, 1 if self.case.startup_first_order_iters < primal.iterations else -1)
        first, done, ratio = None, 0, 1.0
        if self.adjoint_method == "krylov":
            h = s.adjoint_solve_krylov(self.adjoint_max_iters, self.krylov_restart, self.krylov_smooth, cfl,
                                       self.adjoint_tol)
            done, ratio = h.size, (float(h[-1]) if h.size else 0.0)
        else:
            while done < self.adjoint_max_iters:
                n = min(self.chunk, self.adjoint_max_iters - done)
                h = s.adjoint_solve(n, cfl)
                done += n
                if first is None:
                    first = h[0] if h[0] > 0 else 1.0
                ratio = h[-1] / first
                if not np.isfinite(ratio) or ratio < self.adjoint_tol:
                    break
        dalpha = s.adjoint_dalpha()
        if self.geometry_product == "reverse":
            dj_dx = s.adjoint_node_vjp()
            da = np.tensordot(self.modes, dj_dx, axes=([1, 2], [0, 1]))
        else:
            da = np.empty(self.peaks.size)
            for k in range(self.peaks.size):
                da[k] = s.adjoint_geometry(geometry_tangent(primal.mesh, self.modes[k]))
        self.last_adjoint_seconds = time.perf_counter() - t0
        self.last_adjoint_iterations = done
        self.last_adjoint_ratio = float(ratio)
        return da, dalpha


def _torch_function():
    import torch

    class AirfoilForces(torch.autograd.Function):
        """(amplitudes [n], alpha [deg]) -> (CD, CL) through the device solver; backward by the
        discrete adjoint. Call as AirfoilForces.apply(amplitudes, alpha, problem)."""

        @staticmethod
        def forward(ctx, amplitudes, alpha, problem: ShapeProblem):
            a = amplitudes.detach().cpu().double().numpy()
            res = problem.solve(a, float(alpha))
            ctx.problem = problem
            ctx.primal = res
            return torch.tensor([res.cd, res.cl], dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad):
            g = grad.detach().cpu().double().numpy()
            da, dalpha = ctx.problem.gradient(ctx.primal, float(g[0]), float(g[1]))
            return torch.from_numpy(da), torch.tensor(dalpha, dtype=torch.float64), None

    return AirfoilForces


_AIRFOIL_FORCES = None


def __getattr__(name):
    global _AIRFOIL_FORCES
    if name == "AirfoilForces":  # torch is imported on first use only
        if _AIRFOIL_FORCES is None:
            _AIRFOIL_FORCES = _torch_function()
        return _AIRFOIL_FORCES
    raise AttributeError(name)
