"""Discrete adjoint of the FP64 device residual (include/aero_adjoint.h).

No reference counterpart: AeroCFD computes no sensitivities. The checks are the standard
ones for a discrete adjoint:
  * transpose products (dR/dU)^T v against central differences of aero_residual
    (a dot-product test v . dR[d] = (dR^T v) . d over random v, d);
  * dJ/dU of the force coefficients against central differences of the reported CD / CL;
  * dCD/d(alpha), dCL/d(alpha) and dJ/d(Hicks-Henne amplitude) from the converged adjoint
    against central differences of converged FP64 primal solutions.
"""

import numpy as np
import pytest

import aero_gb300
from aero_gb300 import capi
from aero_gb300.adjoint import ShapeProblem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device():
    lib = aero_gb300.load(build_if_missing=True)
    assert lib.aero_cuda_available(), "GPU tests need an sm_103 device"


def _mesh(nc=64, nr=16, seed=3):
    return aero_gb300.ogrid_synthetic(nc, nr, cell_type=3, permute=True, jitter=0.1, seed=seed)


SCHEMES = {
    "rusanov_first": dict(flux=capi.FLUX_RUSANOV, limiter=capi.LIMITER_MINMOD, second=0),
    "hllc_venkat": dict(flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT, second=1),
    "hllc_minmod": dict(flux=capi.FLUX_HLLC, limiter=capi.LIMITER_MINMOD, second=1),
    "rusanov_venkat": dict(flux=capi.FLUX_RUSANOV, limiter=capi.LIMITER_VENKAT, second=1),
}


@pytest.mark.parametrize("scheme", sorted(SCHEMES))
def test_vjp_dot_product_against_residual_differences(scheme):
    """At a developed state with 5% cell-to-cell noise: the limiters' kinks (a b = 0, the
    clamps) sit at zero neighbour differences, which a smooth or near-uniform state has in
    abundance and a 1e-7 perturbation would cross; with O(5%) differences it crosses none,
    and the differenced residual is the derivative of the branches the state takes."""
    sc = SCHEMES[scheme]
    mesh = _mesh()
    case = capi.make_case(mach=0.6, aoa_deg=2.0, flux=sc["flux"], limiter=sc["limiter"], startup_first_order_iters=5,
                          cfl_max=0.8, iterations=100000, precision=capi.PRECISION_FP64)
    with aero_gb300.Solver(mesh, case) as s:
        s.run(150)
        rng = np.random.default_rng(7)
        u = s.get_state() * (1.0 + 0.05 * rng.standard_normal((mesh.num_cells, 5)))
        u[:, 3] = 0.0
        s.set_state(u)
        s.adjoint_linearize(1.0, 0.0, sc["second"])
        scale = np.abs(u).max(axis=0)
        for trial in range(3):
            v = rng.standard_normal(u.shape)
            v[:, 3] = 0.0
            d = rng.standard_normal(u.shape) * scale
            d[:, 3] = 0.0
            eps = 1e-7
            rp, _, _ = s.residual(u + eps * d, second_order=bool(sc["second"]))
            rm, _, _ = s.residual(u - eps * d, second_order=bool(sc["second"]))
            lhs = float(np.sum(v * (rp - rm)) / (2 * eps))
            rhs = float(np.sum(s.adjoint_vjp(v) * d))
            assert abs(lhs - rhs) <= 1e-6 * max(abs(lhs), abs(rhs)), (trial, lhs, rhs)


def test_vjp_is_linear():
    mesh = _mesh(48, 12)
    case = capi.make_case(mach=0.5, aoa_deg=1.0, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT,
                          startup_first_order_iters=5, cfl_max=0.8, iterations=100000)
    with aero_gb300.Solver(mesh, case) as s:
        s.run(100)
        s.adjoint_linearize(0.0, 1.0, 1)
        rng = np.random.default_rng(2)
        a, b = rng.standard_normal((2, mesh.num_cells, 5))
        a[:, 3] = b[:, 3] = 0.0
        np.testing.assert_allclose(s.adjoint_vjp(2.0 * a - 3.0 * b), 2.0 * s.adjoint_vjp(a) - 3.0 * s.adjoint_vjp(b),
                                   rtol=1e-10, atol=1e-12 * np.abs(s.adjoint_vjp(a)).max())
        g = s.adjoint_objective_gradient()
        assert np.abs(g).max() > 0.0 and not g[:, 3].any()


def test_objective_gradient_against_force_differences():
    """dJ/dU of J = 0.3 CD + 0.7 CL against central differences of the gauge-force formula
    (post/forces.cpp:208-294) on perturbed wall-cell states; q S from the run's records."""
    mesh = _mesh(48, 12)
    case = capi.make_case(mach=0.5, aoa_deg=3.0, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT,
                          startup_first_order_iters=5, cfl_max=0.8, iterations=100000)
    with aero_gb300.Solver(mesh, case) as s:
        _, recs = s.run(80)
        u = s.get_state()
        s.adjoint_linearize(0.3, 0.7, 1)
        g = s.adjoint_objective_gradient()
    qs = recs[-1]["drag"] / recs[-1]["cd"]
    gamma = case.gamma

    def force(uu):
        r = np.maximum(uu[:, 0], 1e-8)
        p = np.maximum((gamma - 1) * (uu[:, 4] - 0.5 * (uu[:, 1] ** 2 + uu[:, 2] ** 2) / r), 1e-8)
        f = mesh.wall_faces
        o = mesh.owner[f]
        n = mesh.normal.reshape(-1, 3)[f]
        return np.sum(p[o] * n[:, 0] * mesh.area[f]), np.sum(p[o] * n[:, 1] * mesh.area[f])

    rng = np.random.default_rng(4)
    d = np.zeros_like(u)
    cells = np.unique(mesh.owner[mesh.wall_faces])
    d[cells] = rng.standard_normal((cells.size, 5)) * np.abs(u[cells]).max(axis=0)
    d[:, 3] = 0.0
    eps = 1e-6
    fxp, fyp = force(u + eps * d)
    fxm, fym = force(u - eps * d)
    a = np.deg2rad(3.0)
    dfx, dfy = (fxp - fxm) / (2 * eps), (fyp - fym) / (2 * eps)
    want = (0.3 * (dfx * np.cos(a) + dfy * np.sin(a)) + 0.7 * (-dfx * np.sin(a) + dfy * np.cos(a))) / qs
    got = float(np.sum(g * d))
    assert abs(got - want) <= 1e-6 * abs(want), (got, want)
    # no cell away from the wall contributes
    far = np.setdiff1d(np.arange(mesh.num_cells), cells)
    assert not g[far].any()


def test_adjoint_refuses_fp32_and_unlinearised_contexts():
    mesh = _mesh(32, 8)
    case = capi.make_case(mach=0.5, precision=capi.PRECISION_FP32)
    with aero_gb300.Solver(mesh, case) as s:
        with pytest.raises(aero_gb300.AeroError):
            s.adjoint_linearize(1.0, 0.0)
    with aero_gb300.Solver(mesh, capi.make_case(mach=0.5)) as s:
        with pytest.raises(aero_gb300.AeroError):
            s.adjoint_vjp(np.zeros((mesh.num_cells, 5)))


def _problem(flux, limiter, mach=0.5, nc=64, nr=16):
    mesh = _mesh(nc, nr, seed=11)
    case = capi.make_case(mach=mach, aoa_deg=2.0, flux=flux, limiter=limiter, startup_first_order_iters=20,
                          cfl_max=0.8, precision=capi.PRECISION_FP64)
    return ShapeProblem(mesh, case, peaks=[0.3, 0.6], upper=[1, 0], width=3.0, max_iters=60000, rho_target=1e-13,
                        adjoint_max_iters=60000, adjoint_tol=1e-12)


@pytest.mark.parametrize("scheme", ["rusanov_first", "hllc_venkat"])
def test_gradients_against_converged_differences(scheme):
    sc = SCHEMES[scheme]
    prob = _problem(sc["flux"], sc["limiter"])
    if not sc["second"]:
        prob.case.startup_first_order_iters = 10 ** 9  # first order throughout
    a0 = np.zeros(2)
    base = prob.solve(a0, 2.0)
    assert base.rho_ratio <= 1e-13, base.rho_ratio
    da_cd, dal_cd = prob.gradient(base, 1.0, 0.0)
    assert prob.last_adjoint_ratio <= 1e-12
    da_cl, dal_cl = prob.gradient(base, 0.0, 1.0)

    h_al = 1e-3
    p, m = prob.solve(a0, 2.0 + h_al), prob.solve(a0, 2.0 - h_al)
    fd_cd, fd_cl = (p.cd - m.cd) / (2 * h_al), (p.cl - m.cl) / (2 * h_al)
    assert abs(dal_cd - fd_cd) <= 1e-4 * abs(fd_cd) + 1e-9, (dal_cd, fd_cd)
    assert abs(dal_cl - fd_cl) <= 1e-4 * abs(fd_cl) + 1e-9, (dal_cl, fd_cl)

    h = 1e-5
    for k in range(2):
        e = np.zeros(2)
        e[k] = h
        p, m = prob.solve(e, 2.0), prob.solve(-e, 2.0)
        fd_cd, fd_cl = (p.cd - m.cd) / (2 * h), (p.cl - m.cl) / (2 * h)
        assert abs(da_cd[k] - fd_cd) <= 1e-4 * abs(fd_cd) + 1e-7, (k, da_cd[k], fd_cd)
        assert abs(da_cl[k] - fd_cl) <= 1e-4 * abs(fd_cl) + 1e-7, (k, da_cl[k], fd_cl)


def test_autograd_function_returns_the_adjoint_gradient():
    torch = pytest.importorskip("torch")
    from aero_gb300.adjoint import AirfoilForces

    prob = _problem(capi.FLUX_RUSANOV, capi.LIMITER_MINMOD, nc=48, nr=12)
    a = torch.zeros(2, dtype=torch.float64, requires_grad=True)
    alpha = torch.tensor(2.0, dtype=torch.float64, requires_grad=True)
    out = AirfoilForces.apply(a, alpha, prob)
    (out[0] + 2.0 * out[1]).backward()
    base = prob.solve(np.zeros(2), 2.0)
    assert abs(out[0].item() - base.cd) <= 1e-12 and abs(out[1].item() - base.cl) <= 1e-12
    da, dal = prob.gradient(base, 1.0, 2.0)
    np.testing.assert_allclose(a.grad.numpy(), da, rtol=1e-9, atol=1e-12)
    assert abs(alpha.grad.item() - dal) <= 1e-9 * abs(dal)
