"""Configurations 4 and 5 at their stated sizes.

* Mixed types (the benchmarked mesh: 50^3 cells of the unit cube split into HEX/TET/WEDGE/PYR, 207,312 volumes,
  p uniform in {1,2,3,4}, Roe-Pike, positivity limiter, 41.2 M state values): one residual (at max(1e-12, twice the
  residual's one-ulp noise floor, measured)) and one SSP-RK3 step (at 1e-12) of the batched context in its fused and
  parallel-branch forms against the oracle.
* The discrete adjoint on the curved HEX 32^3 mesh at p = 2 and p = 3 (Lax-Friedrichs): the VJP of R with a seeded
  cotangent against the oracle's complex step (h = 1e-30) and central differences (h = 1e-6), and against the
  GPU's forward-mode JVP on 1000 seeded directions (each a random perturbation of the state of 8 random volumes);
  and the adjoint of 200 SSP-RK3 steps of J = integral of pressure over the z = 0 faces (checkpoints and stage
  recomputation under a 4 GB budget) against central differences of J through 200 forward steps.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_mixed_types_at_stated_size_match_oracle(gpu_lib):
    from dpgsolver_gb300.host.mixed_types import mixed_types_euler
    from dpgsolver_gb300.solver import BatchSimulation
    prob = mixed_types_euler(50, seed=0)
    assert prob.n_volumes == 207312
    o = oracle.Oracle(prob)
    r_ref, mx_ref = o.compute_rhs(prob.sol)
    # volumes 0.02 wide: the residual is a small difference of flux terms. Its noise floor is the oracle's own
    # response to one-ulp input noise, measured here; the residual is held to max(1e-12, 2 x floor)
    noisy = prob.sol * (1.0 + np.random.default_rng(0).choice([-1.0, 1.0], prob.sol.shape) * 2.0 ** -52)
    floor = rel(o.compute_rhs(noisy)[0], r_ref)
    tol = max(1e-12, 2.0 * floor)
    s_ref, _, nc_ref = o.ssp_rk3_step(prob.sol, prob.dt)
    with BatchSimulation(prob) as sim:
        for form in ("fused", "branches", "stage"):
            sim.form = form
            sim.upload_state(prob.sol)
            mx = sim.compute_rhs()
            assert rel(sim.rhs, r_ref) <= tol, (form, rel(sim.rhs, r_ref), floor)
            assert abs(mx - mx_ref) <= tol * mx_ref
            sim.upload_state(prob.sol)
            sim.ssp_rk3_steps(prob.dt, 1)
            assert rel(sim.sol_coef, s_ref) <= 1e-12, form


@pytest.mark.parametrize("p", [2, 3])
def test_adjoint_at_stated_size(gpu_lib, p):
    from dpgsolver_gb300.solver import Simulation
    prob = P.euler_hex_3d(32, p)
    u = prob.sol
    rng = np.random.default_rng(100 + p)
    v = rng.standard_normal(u.shape)
    o = oracle.Oracle(prob)
    with Simulation(prob) as sim:
        sim.vjp_forward(u)
        g = sim.vjp_backward(v)
        # complex step and central differences of the oracle's residual, three seeded dense directions
        for k in range(3):
            d = rng.standard_normal(u.shape)
            _, ri = o.compute_rhs_cmplx(u, 1e-30 * d)
            jd = ri / 1e-30
            lhs, rhs = float(np.sum(g * d)), float(np.sum(v * jd))
            scale = float(np.sum(np.abs(v * jd)))
            assert abs(lhs - rhs) <= 1e-8 * scale, (k, lhs, rhs)
            if k == 0:
                rp, _ = o.compute_rhs(u + 1e-6 * d)
                rm, _ = o.compute_rhs(u - 1e-6 * d)
                fd = float(np.sum(v * (rp - rm) / 2e-6))
                assert abs(lhs - fd) <= 1e-4 * scale
        # 1000 seeded directions against the forward-mode JVP (dual numbers)
        nv = prob.n_volumes
        d = np.zeros(u.shape)
        worst = 0.0
        for k in range(1000):
            vols = rng.choice(nv, size=8, replace=False)
            d[vols] = rng.standard_normal((8,) + u.shape[1:])
            _, jv = sim.jvp(u, d)
            lhs, rhs = float(np.sum(g * d)), float(np.sum(v * jv))
            scale = float(np.sum(np.abs(v * jv)))
            worst = max(worst, abs(lhs - rhs) / scale)
            d[vols] = 0.0
        assert worst <= 1e-10, worst

        # the adjoint of 200 SSP-RK3 steps of J = integral of p over z = 0, against central differences
        sim.set_objective_faces(prob.faces_on_plane(2))
        J, grad, _ = sim.adjoint_ssp_rk3(u, prob.dt, 200, 4 << 30)
        dj = rng.standard_normal(u.shape) * np.abs(u).max(axis=(0, 2), keepdims=True)
        eps = 1e-6

        def j_after(s0):
            sim.upload_state(s0)
            sim.ssp_rk3_steps(prob.dt, 200)
            return sim.objective(sim.sol_coef, gradient=False)
        fd = (j_after(u + eps * dj) - j_after(u - eps * dj)) / (2 * eps)
        lhs = float(np.sum(grad * dj))
        assert abs(lhs - fd) <= 1e-5 * max(abs(fd), 1e-300), (lhs, fd)
