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
from oracle import oracle_py as op

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


def _problem(flux, limiter, mach=0.5, nc=64, nr=16, first_order=False):
    mesh = _mesh(nc, nr, seed=11)
    case = capi.make_case(mach=mach, aoa_deg=2.0, flux=flux, limiter=limiter,
                          startup_first_order_iters=10 ** 9 if first_order else 20, cfl_max=0.8,
                          precision=capi.PRECISION_FP64)
    return ShapeProblem(mesh, case, peaks=[0.3, 0.6], upper=[1, 0], width=3.0, max_iters=60000, rho_target=1e-13,
                        adjoint_max_iters=3000, adjoint_tol=1e-12, adjoint_method="krylov")


def test_gradients_against_converged_differences():
    """End to end on a scheme whose primal converges to round-off (first-order Rusanov; the
    reference's second-order limiters stall the primal at density-residual ratios of 1e-3 on
    these meshes, so converged differences of second-order solutions do not exist)."""
    prob = _problem(capi.FLUX_RUSANOV, capi.LIMITER_MINMOD, first_order=True)
    a0 = np.zeros(2)
    base = prob.solve(a0, 2.0)
    assert base.rho_ratio <= 1e-13, base.rho_ratio
    da_cd, dal_cd = prob.gradient(base, 1.0, 0.0)
    assert prob.last_adjoint_ratio <= 1e-12
    da_cl, dal_cl = prob.gradient(base, 0.0, 1.0)
    prob.adjoint_method = "smoother"  # the plain RK3 iteration converges here too
    prob.adjoint_max_iters = 60000
    da_cd2, dal_cd2 = prob.gradient(base, 1.0, 0.0)
    np.testing.assert_allclose(da_cd2, da_cd, rtol=1e-7)
    assert abs(dal_cd2 - dal_cd) <= 1e-7 * abs(dal_cd)

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


def test_krylov_matches_the_smoother_and_satisfies_the_adjoint_equation():
    """GMRES (preconditioned by smoother sweeps) and the plain RK3 smoother reach the same
    lam on a converged first-order state, and lam satisfies (dR/dU)^T lam + dJ/dU = 0
    through the independent transpose-product call."""
    mesh = _mesh(64, 16, seed=11)
    case = capi.make_case(mach=0.5, aoa_deg=2.0, flux=capi.FLUX_RUSANOV, startup_first_order_iters=10 ** 9,
                          cfl_max=0.8, iterations=100000)
    with aero_gb300.Solver(mesh, case) as s:
        s.run(60000)
        s.adjoint_linearize(1.0, 0.0, 0)
        h = s.adjoint_solve_krylov(max_iters=2000, restart=40, smooth=10, cfl=0.8, rtol=1e-11)
        assert h.size < 2000 and h[-1] <= 1e-11, (h.size, h[-1])
        lam_k = s.adjoint_lambda()
        g = s.adjoint_objective_gradient()
        r = s.adjoint_vjp(lam_k) + g
        assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(g)
        s.adjoint_set_lambda(np.zeros_like(lam_k))
        hs = s.adjoint_solve(40000, 0.8)
        assert hs[-1] <= 1e-9 * hs[0]
        lam_s = s.adjoint_lambda()
        assert np.linalg.norm(lam_s - lam_k) <= 1e-7 * np.linalg.norm(lam_k)


def _wall_force(mesh, u, gamma, p_inf):
    r = np.maximum(u[:, 0], 1e-8)
    p = np.maximum((gamma - 1) * (u[:, 4] - 0.5 * (u[:, 1] ** 2 + u[:, 2] ** 2) / r), 1e-8)
    f = mesh.wall_faces
    n = mesh.normal.reshape(-1, 3)[f]
    dp = p[mesh.owner[f]] - p_inf
    return np.sum(dp * n[:, 0] * mesh.area[f]), np.sum(dp * n[:, 1] * mesh.area[f])


@pytest.mark.parametrize("scheme", ["hllc_venkat", "rusanov_first"])
def test_parameter_partials_against_residual_differences(scheme):
    """lam^T dR/dalpha and lam^T dR/dX . m_k for a random lam, and the explicit force terms
    (lam = 0), against central differences of the residual and of the wall force at a fixed
    state: far-field state at alpha +- h, and meshes deformed by +- h m_k."""
    sc = SCHEMES[scheme]
    mesh = _mesh(48, 12, seed=9)
    mk = dict(mach=0.6, flux=sc["flux"], limiter=sc["limiter"], startup_first_order_iters=5, cfl_max=0.8,
              iterations=100000)
    case = capi.make_case(aoa_deg=2.0, **mk)
    modes = aero_gb300.hicks_henne_modes(mesh, [0.35, 0.7], [1, 0], 3.0)
    pts = mesh.points.reshape(-1, 3)
    second = bool(sc["second"])
    with aero_gb300.Solver(mesh, case) as s:
        _, recs = s.run(200)
        rng = np.random.default_rng(3)
        u = s.get_state() * (1.0 + 0.02 * rng.standard_normal((mesh.num_cells, 5)))
        u[:, 3] = 0.0
        s.set_state(u)
        s.adjoint_linearize(0.4, 0.6, sc["second"])
        lam = rng.standard_normal((mesh.num_cells, 5))
        lam[:, 3] = 0.0
        s.adjoint_set_lambda(np.zeros_like(lam))
        d0 = s.adjoint_dalpha()
        g0 = [s.adjoint_geometry(aero_gb300.geometry_tangent(mesh, modes[k])) for k in range(2)]
        s.adjoint_set_lambda(lam)
        d1 = s.adjoint_dalpha()
        g1 = [s.adjoint_geometry(aero_gb300.geometry_tangent(mesh, modes[k])) for k in range(2)]
    qs = recs[-1]["drag"] / recs[-1]["cd"]
    gamma, p_inf = case.gamma, case.p_inf

    def J(m, alpha):
        fx, fy = _wall_force(m, u, gamma, p_inf)
        a = np.deg2rad(alpha)
        return (0.4 * (fx * np.cos(a) + fy * np.sin(a)) + 0.6 * (-fx * np.sin(a) + fy * np.cos(a))) / qs

    def R(m, alpha):
        c = capi.make_case(**mk)
        c.aoa_deg = alpha  # exact, not rounded to float like a case-file value
        with aero_gb300.Solver(m, c) as t:
            return t.residual(u, second_order=second)[0]

    # incidence (per degree); the far-field state is the only residual input that moves
    h = 1e-4
    fd_exp = (J(mesh, 2.0 + h) - J(mesh, 2.0 - h)) / (2 * h)
    assert abs(d0 - fd_exp) <= 1e-7 * abs(fd_exp), (d0, fd_exp)
    fd_lam = np.sum(lam * (R(mesh, 2.0 + h) - R(mesh, 2.0 - h))) / (2 * h)
    assert abs((d1 - d0) - fd_lam) <= 1e-6 * abs(fd_lam), (d1 - d0, fd_lam)
    # shape modes (case aoa is the float-rounded 2.0 for both meshes)
    hx = 1e-6
    for k in range(2):
        mp = aero_gb300.deform(mesh, pts + hx * modes[k])
        mm = aero_gb300.deform(mesh, pts - hx * modes[k])
        fd_exp = (J(mp, 2.0) - J(mm, 2.0)) / (2 * hx)
        assert abs(g0[k] - fd_exp) <= 1e-6 * abs(fd_exp) + 1e-9, (k, g0[k], fd_exp)
        fd_lam = np.sum(lam * (R(mp, 2.0) - R(mm, 2.0))) / (2 * hx)
        assert abs((g1[k] - g0[k]) - fd_lam) <= 1e-5 * abs(fd_lam), (k, g1[k] - g0[k], fd_lam)


def test_autograd_function_returns_the_adjoint_gradient():
    torch = pytest.importorskip("torch")
    from aero_gb300.adjoint import AirfoilForces

    prob = _problem(capi.FLUX_RUSANOV, capi.LIMITER_MINMOD, nc=48, nr=12, first_order=True)
    a = torch.zeros(2, dtype=torch.float64, requires_grad=True)
    alpha = torch.tensor(2.0, dtype=torch.float64, requires_grad=True)
    out = AirfoilForces.apply(a, alpha, prob)
    (out[0] + 2.0 * out[1]).backward()
    base = prob.solve(np.zeros(2), 2.0)
    assert abs(out[0].item() - base.cd) <= 1e-12 and abs(out[1].item() - base.cl) <= 1e-12
    da, dal = prob.gradient(base, 1.0, 2.0)
    np.testing.assert_allclose(a.grad.numpy(), da, rtol=1e-9, atol=1e-12)
    assert abs(alpha.grad.item() - dal) <= 1e-9 * abs(dal)


def _oracle_cd(prim, alpha_deg, iters=60):
    """CD of a converged device state as the FP64 oracle computes it on the same deformed mesh
    after `iters` further iterations started from that state, with the oracle's own density
    residual over them (the state must already be the oracle's steady state)."""
    from aero_gb300.adjoint import converged_case

    case = converged_case(prim.solver.case, alpha_deg, capi.PRECISION_FP64, iters, 0.0)
    o = op.OracleSolver(op.MODE_DOUBLE, prim.mesh, case)
    o.set_state(prim.solver.get_state())
    _, rec = o.run(iters)
    return float(rec["cd"][-1]), rec


def test_gradients_against_oracle_central_differences():
    """The adjoint configuration's numerics (HLLC, M = 0.75, alpha = 2 deg, 16 Hicks-Henne bumps
    with the configuration's seeded draw, J = CD, first order: the second-order primal has no
    steady state on these meshes) on the 64x16 grid of its family. dCD/dalpha and dCD/da_0 from
    the discrete adjoint against central differences (step 1e-6) of CD from the FP64 CPU oracle:
    each perturbed state is converged on the device to a density-residual ratio of 1e-13, then
    handed to the oracle, which must keep it (its own residual stays at round-off) and
    integrates CD from it. Agreement within 1e-4 relative."""
    op.build()
    rng = np.random.default_rng(5)
    peaks = rng.uniform(0.05, 0.95, 16)
    upper = np.array([1] * 8 + [0] * 8)
    amps = rng.normal(0.0, 1e-3, 16)
    mesh = aero_gb300.ogrid_synthetic(64, 16, cell_type=3, permute=True, jitter=0.1, seed=55)
    case = capi.make_case(mach=0.75, aoa_deg=2.0, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_VENKAT,
                          startup_first_order_iters=10 ** 9, cfl_start=0.2, cfl_max=0.8, cfl_ramp_iters=120,
                          precision=capi.PRECISION_FP64)
    prob = ShapeProblem(mesh, case, peaks=peaks, upper=upper, width=3.0, max_iters=200000, rho_target=1e-13,
                        chunk=20000, adjoint_max_iters=400000, adjoint_tol=1e-12, adjoint_method="smoother")
    base = prob.solve(amps, 2.0)
    assert base.rho_ratio <= 1e-13
    da, dal = prob.gradient(base, 1.0, 0.0)
    assert prob.last_adjoint_ratio <= 1e-12
    cd0, _ = _oracle_cd(base, 2.0)
    assert abs(cd0 - base.cd) <= 1e-12 * abs(base.cd)  # the oracle agrees on the base state's CD
    # the oracle's residual at the free stream, the scale its residual at a steady state is read against
    _, fs = op.OracleSolver(op.MODE_DOUBLE, base.mesh, case).run(1)
    l2_free = float(fs["residual_l2"][0])
    h = 1e-6
    for name, e, al in (("alpha", np.zeros(16), h), ("a0", np.eye(16)[0] * h, 0.0)):
        cds = []
        for sgn in (1.0, -1.0):
            prim = prob.solve(amps + sgn * e, 2.0 + sgn * al)
            assert prim.rho_ratio <= 1e-13
            cd, rec = _oracle_cd(prim, 2.0 + sgn * al)
            # the device state is the oracle's steady state: its residual stays at round-off
            assert rec["residual_l2"][-1] <= 1e-11 * l2_free
            cds.append(cd)
            prim.solver.close()
        fd = (cds[0] - cds[1]) / (2 * h)
        adj = dal if name == "alpha" else float(da[0])
        assert abs(adj - fd) <= 1e-4 * abs(fd), (name, adj, fd)


@pytest.mark.parametrize("scheme", sorted(SCHEMES))
@pytest.mark.parametrize("low_mach", [False, True])
def test_geometry_vjp_is_the_transpose_of_the_geometry_product(scheme, low_mach):
    """The reverse geometry product (one pass for every face normal, length and centre and
    every cell volume and centre) against the forward one: for random lam and random node
    displacements dX, sum(vjp * tangent(dX)) = lam^T dR/dX dX + dJ/dX|_U dX from
    aero_adjoint_geometry, and the node-level product sum(dJ/dX * dX) gives the same number."""
    sc = SCHEMES[scheme]
    mesh = _mesh(48, 12, seed=9)
    kw = dict(mach=0.6, aoa_deg=2.0, flux=sc["flux"], limiter=sc["limiter"], startup_first_order_iters=5,
              cfl_max=0.8, iterations=100000, precision=capi.PRECISION_FP64)
    if low_mach:
        kw.update(mach=0.2, precond_on=1, low_mach_fix=1, all_speed_flux_fix=1, precond_farfield_bc=1)
    case = capi.make_case(**kw)
    rng = np.random.default_rng(11)
    with aero_gb300.Solver(mesh, case) as s:
        s.run(60)
        s.adjoint_linearize(0.7, 0.3, sc["second"])
        lam = rng.standard_normal((mesh.num_cells, 5))
        lam[:, 3] = 0.0
        s.adjoint_set_lambda(lam)
        bars = s.adjoint_geometry_vjp()
        nodes = s.adjoint_node_vjp()
        pts = mesh.points.reshape(-1, 3)
        for trial in range(3):
            dp = np.zeros_like(pts)
            dp[:, :2] = rng.standard_normal((pts.shape[0], 2)) * 1e-3
            t = aero_gb300.geometry_tangent(mesh, dp)
            want = s.adjoint_geometry(t)
            got = sum(float(np.dot(getattr(bars, k), getattr(t, k)))
                      for k in ("normal", "center", "area", "volume", "cell_center"))
            assert abs(got - want) <= 1e-10 * abs(want), (trial, got, want)
            assert abs(float(np.sum(nodes * dp)) - want) <= 1e-10 * abs(want), trial


def test_shape_gradient_by_the_node_reverse_product():
    """ShapeProblem's gradient through dJ/dX (one reverse pass, then the modes) equals the one
    through one geometry tangent per bump."""
    mesh = _mesh(64, 16, seed=11)
    case = capi.make_case(mach=0.5, aoa_deg=2.0, flux=capi.FLUX_HLLC, startup_first_order_iters=10 ** 9,
                          cfl_max=0.8, precision=capi.PRECISION_FP64)
    prob = ShapeProblem(mesh, case, peaks=[0.2, 0.4, 0.6, 0.8], upper=[1, 0, 1, 0], width=3.0, max_iters=100000,
                        rho_target=1e-12, adjoint_max_iters=200000, adjoint_tol=1e-11, adjoint_method="smoother")
    base = prob.solve(np.full(4, 1e-3), 2.0)
    da_t, dal_t = prob.gradient(base, 1.0, 0.5)
    prob.geometry_product = "reverse"
    da_r, dal_r = prob.gradient(base, 1.0, 0.5)
    np.testing.assert_allclose(da_r, da_t, rtol=1e-9, atol=1e-12 * np.abs(da_t).max())
    assert dal_r == dal_t
