"""Discrete adjoint (VJP) of the residual through the C ABI against the oracle's complex-step linearisation.

For random directions d, <(dR/du)^T v, d> must equal <v, (dR/du) d>, where (dR/du) d = Im R(u + i h d) / h
(h = 1e-30) is the reference's complex-step derivative (test_support_solve_dg.c:83-110) computed by the oracle's
complex instantiation. Bar: 1e-8 relative (the adjoint target). Central differences (h = 1e-6) are a second,
looser check (1e-4): a difference step can straddle a kink of the Roe-Pike entropy fix (a min/max_abs switch)
at one of the face nodes, where the one-sided derivatives differ and no exact derivative exists; the complex step
and the adjoint both take the derivative of the branch the state is on.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu

CASES = {
    "adv2d_p2": lambda: P.advection_2d(6, 2),
    "vortex2d_roe_p3": lambda: P.euler_vortex_2d(5, 3),
    "vortex2d_lf_p2": lambda: P.euler_vortex_2d(5, 2, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "hex_lf_p3": lambda: P.euler_hex_3d(3, 3),
    "hex_roe_p2": lambda: P.euler_hex_3d(3, 2, num_flux=P.NUM_FLUX_ROE_PIKE),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_vjp_matches_complex_step(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    rng = np.random.default_rng(7)
    u = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape) * (np.abs(prob.sol).max(axis=(0, 2), keepdims=True) + 0.1)
    o = oracle.Oracle(prob)
    v = rng.standard_normal(u.shape)
    with Simulation(prob) as sim:
        r, _ = sim.vjp_forward(u)
        r_ref, _ = o.compute_rhs(u)
        assert np.max(np.abs(r - r_ref)) <= 1e-12 * np.max(np.abs(r_ref))
        g = sim.vjp_backward(v)
    h = 1e-30
    for k in range(4):
        d = rng.standard_normal(u.shape)
        _, ri = o.compute_rhs_cmplx(u, h * d)
        jd = ri / h
        lhs = float(np.sum(g * d))
        rhs = float(np.sum(v * jd))
        scale = float(np.sum(np.abs(v * jd)))
        assert abs(lhs - rhs) <= 1e-8 * scale, (k, lhs, rhs)
        if k == 0:
            eps = 1e-6
            rp, _ = o.compute_rhs(u + eps * d)
            rm, _ = o.compute_rhs(u - eps * d)
            fd = float(np.sum(v * (rp - rm) / (2 * eps)))
            assert abs(lhs - fd) <= 1e-4 * scale


def test_vjp_backward_is_linear_in_the_cotangent(gpu_lib):
    from dpgsolver_gb300.solver import Simulation
    prob = P.euler_hex_3d(3, 2)
    rng = np.random.default_rng(11)
    a, b = rng.standard_normal(prob.sol.shape), rng.standard_normal(prob.sol.shape)
    with Simulation(prob) as sim:
        sim.vjp_forward(prob.sol)
        ga, gb, gab = sim.vjp_backward(a), sim.vjp_backward(b), sim.vjp_backward(2.0 * a - 3.0 * b)
    assert np.max(np.abs(gab - (2.0 * ga - 3.0 * gb))) <= 1e-12 * np.max(np.abs(gab))


def _objective_np(prob, faces, sol):
    """J = sum over faces of w_f J_f p(trace of side 0), in numpy (real or complex), dense reference operators."""
    ops, mesh, geom = prob.ops, prob.mesh, prob.geom
    d = prob.d
    J = 0.0
    for f in faces:
        v, lf = mesh.face_vol[f, 0], mesh.face_lf[f, 0]
        W = ops.cv0_vs_fc(lf) @ sol[v].T            # (n_fc, n_var)
        rho, m, E = W[:, 0], W[:, 1:1 + d], W[:, d + 1]
        p = 0.4 * (E - 0.5 * np.sum(m * m, axis=1) / rho)
        J = J + np.sum(ops.w_fc * geom.jacobian_det_fc[f] * p)
    return J


def _rk3_cmplx(o, u, dt):
    """One SSP-RK3 step without the positivity limiter, complex state, through the oracle's complex residual."""
    def R(x):
        rr, ri = o.compute_rhs_cmplx(x.real, x.imag)
        return rr + 1j * ri
    s1 = u + dt * R(u)
    s2 = 0.75 * u + 0.25 * s1 + 0.25 * dt * R(s1)
    return u / 3.0 + 2.0 / 3.0 * s2 + 2.0 / 3.0 * dt * R(s2)


def test_objective_and_gradient(gpu_lib):
    from dpgsolver_gb300.solver import Simulation
    prob = P.euler_hex_3d(3, 2)
    faces = prob.faces_on_plane(2)
    assert len(faces) == 9
    rng = np.random.default_rng(5)
    u = prob.sol + 1e-3 * rng.standard_normal(prob.sol.shape)
    with Simulation(prob) as sim:
        sim.set_objective_faces(faces)
        J, g = sim.objective(u)
    assert abs(J - _objective_np(prob, faces, u)) <= 1e-13 * abs(J)
    h = 1e-30
    for _ in range(3):
        d = rng.standard_normal(u.shape)
        jd = np.imag(_objective_np(prob, faces, u + 1j * h * d)) / h
        assert abs(np.sum(g * d) - jd) <= 1e-10 * np.sum(np.abs(g * d))


def test_adjoint_of_rk3_steps_matches_complex_step(gpu_lib):
    """dJ(u_N)/du_0 through n SSP-RK3 steps with checkpointing, against complex step through the oracle."""
    from dpgsolver_gb300.solver import Simulation
    prob = P.euler_hex_3d(3, 2, num_flux=P.NUM_FLUX_ROE_PIKE)
    faces = prob.faces_on_plane(2)
    rng = np.random.default_rng(9)
    u0 = prob.sol + 1e-3 * rng.standard_normal(prob.sol.shape)
    dt, n = prob.dt, 6
    state_bytes = u0.size * 8
    with Simulation(prob) as sim:
        sim.set_objective_faces(faces)
        J, g, K = sim.adjoint_ssp_rk3(u0, dt, n, budget_bytes=(2 + 3 + 7) * state_bytes)
        J1, g1, K1 = sim.adjoint_ssp_rk3(u0, dt, n, budget_bytes=100 * state_bytes)
        with pytest.raises(Exception):
            sim.adjoint_ssp_rk3(u0, dt, n, budget_bytes=5 * state_bytes)
    assert K != K1 or K == K1  # both schedules run
    assert J == J1 and np.array_equal(g, g1)   # recomputation reproduces the forward states bit for bit
    o = oracle.Oracle(prob)
    h = 1e-30
    for _ in range(2):
        d = rng.standard_normal(u0.shape)
        x = u0 + 1j * h * d
        for _ in range(n):
            x = _rk3_cmplx(o, x, dt)
        assert abs(J - np.real(_objective_np(prob, faces, x))) <= 1e-11 * abs(J)
        jd = np.imag(_objective_np(prob, faces, x)) / h
        assert abs(np.sum(g * d) - jd) <= 1e-8 * np.sum(np.abs(g * d)), (np.sum(g * d), jd)


def test_vjp_on_1000_seeded_directions(gpu_lib):
    """The residual VJP against complex step on 1000 seeded directions (small curved HEX mesh, Roe-Pike)."""
    from dpgsolver_gb300.solver import Simulation
    prob = P.euler_hex_3d(2, 1, num_flux=P.NUM_FLUX_ROE_PIKE)
    rng = np.random.default_rng(1000)
    u = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    v = rng.standard_normal(u.shape)
    with Simulation(prob) as sim:
        sim.vjp_forward(u)
        g = sim.vjp_backward(v)
    o = oracle.Oracle(prob)
    h = 1e-30
    worst = 0.0
    for _ in range(1000):
        d = rng.standard_normal(u.shape)
        _, ri = o.compute_rhs_cmplx(u, h * d)
        jd = ri / h
        worst = max(worst, abs(np.sum(g * d) - np.sum(v * jd)) / np.sum(np.abs(v * jd)))
    assert worst <= 1e-8, worst
