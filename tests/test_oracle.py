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


# ---- mixed-order meshes (p per volume, faces at p_f = max(p_L, p_R)) ----------------------------------------------

def _mixed_cases():
    from dpgsolver_gb300.host import mixed as M
    return [lambda: M.mixed_euler(3, 3, seed=0), lambda: M.mixed_euler(2, 5, seed=1),
            lambda: M.mixed_advection_2d(5), lambda: M.mixed_vortex_2d(5),
            lambda: M.mixed_ns(2, 4, seed=2), lambda: M.mixed_ns(3, 3, seed=3, curved=True)]


@pytest.mark.parametrize("k", range(6))
def test_mixed_conservation(k):
    """Face fluxes at p_f telescope across volumes of different p: the sum of raw residuals vanishes."""
    prob = _mixed_cases()[k]()
    o = oracle.Oracle(prob)
    raw = o.compute_rhs_raw(prob.sol)
    tot = np.zeros(prob.n_var)
    scale = np.zeros(prob.n_var)
    for v in range(prob.n_volumes):
        b = prob.block(raw, v)
        tot += b.sum(axis=1)
        scale += np.abs(b).sum(axis=1)
    assert np.all(np.abs(tot) <= 1e-13 * scale.max())


def test_mixed_free_stream_on_straight_mesh():
    from dpgsolver_gb300.host import mixed as M
    prob = M.mixed_euler(3, 3, seed=0)
    s = prob.sol.copy()
    for v in range(prob.n_volumes):
        b = prob.block(s, v)
        for j, val in enumerate([1.0, 0.3, -0.2, 0.1, 2.5]):
            b[j] = val
    _, mx = oracle.Oracle(prob).compute_rhs(s)
    assert mx < 1e-11


def test_mixed_layout():
    from dpgsolver_gb300.host import mixed as M
    prob = M.mixed_euler(3, 4, seed=0)
    fl = prob.flat()
    q = np.array([prob.groups[g].q for g in prob.vol_group])
    assert fl["sol"].size == np.sum(5 * q ** 3)
    assert fl["metrics_vc"].size == np.sum(9 * q ** 3)
    assert np.array_equal(prob.face_q, np.maximum(q[prob.mesh.face_vol[:, 0]], q[prob.mesh.face_vol[:, 1]]))
    assert fl["jacobian_det_fc"].size == np.sum(prob.face_q.astype(np.int64) ** 2)
    assert sorted(set(int(p) for p in prob.p_vol)) == [1, 2, 3, 4]


def test_mixed_complex_step_matches_central_differences():
    from dpgsolver_gb300.host import mixed as M
    prob = M.mixed_euler(3, 3, seed=0)
    o = oracle.Oracle(prob)
    rng = np.random.default_rng(2)
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    dirn = rng.standard_normal(prob.sol.shape)
    h = 1e-30
    _, ri = o.compute_rhs_cmplx(base, h * dirn)
    eps = 1e-6
    jv_fd = (o.compute_rhs(base + eps * dirn)[0] - o.compute_rhs(base - eps * dirn)[0]) / (2 * eps)
    assert np.max(np.abs(ri / h - jv_fd)) <= 1e-6 * np.max(np.abs(ri / h))
