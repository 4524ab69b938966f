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
