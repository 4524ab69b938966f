"""The CPU oracle against the known-answer properties the reference's tests pin for this path."""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import problem as P


def _euler_const(prob):
    vals = [1.0, 0.3, -0.2] + ([0.1] if prob.d == 3 else []) + [2.5]
    return P.constant_state(prob, vals)


@pytest.mark.parametrize("mk", [lambda: P.euler_vortex_2d(6, 3), lambda: P.euler_hex_3d(3, 2),
                                lambda: P.euler_hex_3d(3, 3, num_flux=P.NUM_FLUX_ROE_PIKE)])
def test_free_stream_preservation(mk):
    """Residual of a constant state vanishes on curved meshes (test_integration_free_stream.c:52-86)."""
    prob = mk()
    o = oracle.Oracle(prob)
    _, mx = o.compute_rhs(_euler_const(prob))
    assert mx < 1e-11


@pytest.mark.parametrize("mk", [lambda: P.advection_2d(6, 2), lambda: P.euler_vortex_2d(5, 3),
                                lambda: P.euler_hex_3d(3, 2)])
def test_conservation(mk):
    """Periodic mesh: sum over volumes of 1^T M R = sum of raw residuals vanishes (telescoping face fluxes)."""
    prob = mk()
    o = oracle.Oracle(prob)
    raw = o.compute_rhs_raw(prob.sol)
    tot = raw.sum(axis=(0, 2))
    scale = np.abs(raw).sum(axis=(0, 2))
    assert np.all(np.abs(tot) <= 1e-13 * scale.max())


def test_mass_inverse():
    prob = P.euler_vortex_2d(3, 3)
    o = oracle.Oracle(prob)
    ops = prob.ops
    V = ops.cv0_vs_vc()
    for v in range(prob.n_volumes):
        M = V.T @ np.diag(ops.w_vc * prob.geom.jacobian_det_vc[v]) @ V
        assert np.max(np.abs(o.m_inv(v) @ M - np.eye(ops.n_vs))) < 1e-11


def test_advection_residual_is_linear():
    prob = P.advection_2d(5, 3)
    o = oracle.Oracle(prob)
    rng = np.random.default_rng(0)
    a, b = rng.standard_normal(prob.sol.shape), rng.standard_normal(prob.sol.shape)
    ra, _ = o.compute_rhs(a)
    rb, _ = o.compute_rhs(b)
    rab, _ = o.compute_rhs(2.0 * a - 0.5 * b)
    assert np.max(np.abs(rab - (2.0 * ra - 0.5 * rb))) < 1e-12 * np.max(np.abs(rab))


def test_advection_exact_derivative_of_smooth_solution():
    """Residual approximates -b.grad(u) with spectral accuracy (the convergence property of
    test_integration_convergence.c)."""
    errs = []
    for n in (4, 8):
        prob = P.advection_2d(n, 3)
        o = oracle.Oracle(prob)
        r, _ = o.compute_rhs(prob.sol)
        xyz = prob.solution_node_xyz()
        x, y = xyz[..., 0], xyz[..., 1]
        exact = -(1.0 * np.pi * np.cos(np.pi * x) * np.sin(np.pi * y) + 0.5 * np.pi * np.sin(np.pi * x) * np.cos(np.pi * y))
        errs.append(np.max(np.abs(r[:, 0, :] - exact)))
    assert errs[1] < errs[0] / 6.0


@pytest.mark.parametrize("mk", [lambda: P.euler_vortex_2d(4, 2), lambda: P.euler_hex_3d(2, 2, num_flux=P.NUM_FLUX_ROE_PIKE)])
def test_complex_step_matches_central_differences(mk):
    """The complex instantiation (the reference's complex-step linearisation, test_support_solve_dg.c:83-110)
    gives the directional derivative that central finite differences approximate."""
    prob = mk()
    o = oracle.Oracle(prob)
    rng = np.random.default_rng(1)
    # Additive, element-discontinuous perturbation: it keeps the state away from the kinks of the Roe-Pike
    # entropy fix (|Vn| at Vn = 0, min/max_abs ties when both traces agree), where complex step and central
    # differences legitimately disagree.
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    dirn = rng.standard_normal(prob.sol.shape)
    h = 1e-30
    _, ri = o.compute_rhs_cmplx(base, h * dirn)
    jv_cs = ri / h
    eps = 1e-6
    rp, _ = o.compute_rhs(base + eps * dirn)
    rm, _ = o.compute_rhs(base - eps * dirn)
    jv_fd = (rp - rm) / (2 * eps)
    assert np.max(np.abs(jv_cs - jv_fd)) <= 1e-6 * np.max(np.abs(jv_cs))
    rr, _ = o.compute_rhs_cmplx(base, h * dirn)
    r0, _ = o.compute_rhs(base)
    assert np.max(np.abs(rr - r0)) <= 1e-13 * np.max(np.abs(r0))


def test_positivity_correction_restores_bezier_bounds():
    prob = P.euler_vortex_2d(4, 2)
    sol = prob.sol.copy()
    v, n = 5, 4
    scale = 1e-14 / sol[v, 0, n]
    sol[v, :3, n] *= scale
    o = oracle.Oracle(prob)
    s, ncorr = o.enforce_positivity(sol)
    assert ncorr == 1
    SB = prob.ops.ccSB0_vs_vs()
    rho_b = SB @ s[v, 0, :]
    assert rho_b.min() >= 1e-13 * (1 - 1e-6)
    # untouched volumes are unchanged up to the round trip
    assert np.max(np.abs(s[0] - sol[0])) < 1e-14


def test_rk3_step_consistent_with_residual():
    """For a linear residual one SSP-RK3 step equals the third-order Taylor polynomial in dt R."""
    prob = P.advection_2d(4, 2)
    o = oracle.Oracle(prob)
    dt = prob.dt
    u = prob.sol
    s, _, _ = o.ssp_rk3_step(u, dt)
    r1, _ = o.compute_rhs(u)
    r2, _ = o.compute_rhs(r1)
    r3, _ = o.compute_rhs(r2)
    taylor = u + dt * r1 + dt ** 2 / 2 * r2 + dt ** 3 / 6 * r3
    assert np.max(np.abs(s - taylor)) < 1e-13
