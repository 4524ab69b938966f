"""Discrete adjoint of the Navier-Stokes residual (BR2 gradients, liftings, viscous flux, wall boundary values)
through the C ABI, against the oracle's complex-step linearisation of its restatement of the reference's data flow.

For seeded directions d, <(dR/du)^T v, d> must equal <v, (dR/du) d> with (dR/du) d = Im R(u + i h d) / h (h = 1e-30,
the reference's complex step, test_support_solve_dg.c:83-110), at 1e-8 relative as the Euler adjoint. Also: the VJP
is linear in the cotangent and is the transpose of the GPU's own forward-mode JVP; the objective's gradient and the
checkpointed adjoint of SSP-RK3 steps match complex step through the oracle, as for Euler.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu

CASES = {
    "vortex2d_roe_p3_5": lambda: P.ns_vortex_2d(5, 3, mu=0.02),
    "vortex2d_lf_p2_4": lambda: P.ns_vortex_2d(4, 2, mu=0.05, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "vortex2d_suth_p4_3": lambda: P.ns_vortex_2d(3, 4, mu=0.05, viscosity=P.VISCOSITY_SUTHERLAND),
    "tgv_p3_3_curved": lambda: P.ns_taylor_green(3, 3, Re=100.0, mach=0.3, amplitude=0.1),
    "tgv_p2_3_lf_suth": lambda: P.ns_taylor_green(3, 2, Re=200.0, mach=0.3, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS,
                                                   viscosity=P.VISCOSITY_SUTHERLAND),
    # walls and Riemann sides
    "channel2d_roe_p3_4": lambda: P.ns_channel(2, 4, 3, mu=0.02, amplitude=0.05),
    "channel3d_lf_p2_3": lambda: P.ns_channel(3, 3, 2, mu=0.02, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "riemann2d_roe_p3_4": lambda: P.ns_riemann_vortex_2d(4, 3, mu=0.02),
    # rotating inner wall; adiabatic or diabatic outer wall
    "couette_roe_p3_4": lambda: P.ns_taylor_couette(4, 3, mu=0.02, perturb=0.2),
    "couette_diab_lf_p2_4": lambda: P.ns_taylor_couette(4, 2, mu=0.02, diabatic=True, perturb=0.2,
                                                         num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
}


def _perturbed(prob, rng, scale=1e-2):
    mag = np.abs(prob.sol).max(axis=(0, 2), keepdims=True) + 0.1
    return prob.sol + scale * rng.standard_normal(prob.sol.shape) * mag


@pytest.mark.parametrize("name", sorted(CASES))
def test_ns_vjp_matches_complex_step(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    rng = np.random.default_rng(17)
    u = _perturbed(prob, rng)
    o = oracle.Oracle(prob)
    v = rng.standard_normal(u.shape)
    with Simulation(prob) as sim:
        r, _ = sim.vjp_forward(u)
        r_ref, _ = o.compute_rhs(u)
        assert np.max(np.abs(r - r_ref)) <= 1e-10 * np.max(np.abs(r_ref))
        g = sim.vjp_backward(v)
    h = 1e-30
    for k in range(3):
        d = rng.standard_normal(u.shape)
        _, ri = o.compute_rhs_cmplx(u, h * d)
        jd = ri / h
        lhs, rhs = float(np.sum(g * d)), float(np.sum(v * jd))
        scale = float(np.sum(np.abs(v * jd)))
        assert abs(lhs - rhs) <= 1e-8 * scale, (k, lhs, rhs)


@pytest.mark.parametrize("name", ["tgv_p3_3_curved", "couette_roe_p3_4"])
def test_ns_vjp_is_the_transpose_of_the_jvp_and_linear(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    rng = np.random.default_rng(23)
    u = _perturbed(prob, rng)
    a, b = rng.standard_normal(u.shape), rng.standard_normal(u.shape)
    with Simulation(prob) as sim:
        sim.vjp_forward(u)
        ga, gb, gab = sim.vjp_backward(a), sim.vjp_backward(b), sim.vjp_backward(2.0 * a - 3.0 * b)
        assert np.max(np.abs(gab - (2.0 * ga - 3.0 * gb))) <= 1e-12 * np.max(np.abs(gab))
        worst = 0.0
        for _ in range(20):
            d = rng.standard_normal(u.shape)
            _, jv = sim.jvp(u, d)
            lhs, rhs = float(np.sum(ga * d)), float(np.sum(a * jv))
            worst = max(worst, abs(lhs - rhs) / float(np.sum(np.abs(a * jv))))
    assert worst <= 1e-10, worst


def _objective_np(prob, faces, sol):
    """J = sum over faces of w_f J_f p(trace of side 0), in numpy (real or complex), dense reference operators."""
    ops, mesh, geom = prob.ops, prob.mesh, prob.geom
    d = prob.d
    J = 0.0
    for f in faces:
        v, lf = mesh.face_vol[f, 0], mesh.face_lf[f, 0]
        W = ops.cv0_vs_fc(lf) @ sol[v].T
        rho, m, E = W[:, 0], W[:, 1:1 + d], W[:, d + 1]
        p = 0.4 * (E - 0.5 * np.sum(m * m, axis=1) / rho)
        J = J + np.sum(ops.w_fc * geom.jacobian_det_fc[f] * p)
    return J


def _rk3_cmplx(o, u, dt):
    def R(x):
        rr, ri = o.compute_rhs_cmplx(x.real, x.imag)
        return rr + 1j * ri
    s1 = u + dt * R(u)
    s2 = 0.75 * u + 0.25 * s1 + 0.25 * dt * R(s1)
    return u / 3.0 + 2.0 / 3.0 * s2 + 2.0 / 3.0 * dt * R(s2)


def test_ns_adjoint_of_rk3_steps_matches_complex_step(gpu_lib):
    """dJ(u_N)/du_0 of the pressure integral over z = 0 through 4 SSP-RK3 steps of the curved Taylor-Green vortex,
    against complex step through the oracle; the objective and its gradient alone as well."""
    from dpgsolver_gb300.solver import Simulation
    prob = P.ns_taylor_green(3, 2, Re=100.0, mach=0.3, amplitude=0.1)
    faces = prob.faces_on_plane(2)
    rng = np.random.default_rng(29)
    u0 = _perturbed(prob, rng, 1e-3)
    dt, n = prob.dt, 4
    o = oracle.Oracle(prob)
    h = 1e-30
    with Simulation(prob) as sim:
        sim.set_objective_faces(faces)
        J0, g0 = sim.objective(u0)
        assert abs(J0 - _objective_np(prob, faces, u0)) <= 1e-13 * abs(J0)
        d = rng.standard_normal(u0.shape)
        jd = np.imag(_objective_np(prob, faces, u0 + 1j * h * d)) / h
        assert abs(np.sum(g0 * d) - jd) <= 1e-10 * np.sum(np.abs(g0 * d))
        J, g, _ = sim.adjoint_ssp_rk3(u0, dt, n, budget_bytes=64 * u0.size * 8)
    for _ in range(2):
        d = rng.standard_normal(u0.shape)
        x = u0 + 1j * h * d
        for _ in range(n):
            x = _rk3_cmplx(o, x, dt)
        assert abs(J - np.real(_objective_np(prob, faces, x))) <= 1e-11 * abs(J)
        jd = np.imag(_objective_np(prob, faces, x)) / h
        assert abs(np.sum(g * d) - jd) <= 1e-8 * np.sum(np.abs(g * d)), (np.sum(g * d), jd)
