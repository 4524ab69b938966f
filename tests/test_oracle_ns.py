"""The oracle's Navier-Stokes residual (Euler flux + viscous flux with BR2 gradients) against known answers.

The reference has no golden vectors for this path; its Navier-Stokes tests are convergence runs. Pinned here:
with mu = 0 the residual is the Euler residual bit for bit; the viscous part is linear in mu (constant viscosity);
a constant state is steady; every conserved variable is conserved on a periodic mesh; the complex instantiation
agrees with central differences; and the viscous part converges to the analytic divergence of the viscous flux at
the solution nodes at the rate h^(p-1) expected of a second-order operator's nodal residual.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import problem as P

PR = 0.72


def test_zero_viscosity_is_the_euler_residual():
    r_ns, _ = oracle.Oracle(P.ns_vortex_2d(4, 3, mu=0.0)).compute_rhs(P.ns_vortex_2d(4, 3, mu=0.0).sol)
    pe = P.euler_vortex_2d(4, 3)
    r_e, _ = oracle.Oracle(pe).compute_rhs(pe.sol)
    assert np.array_equal(r_ns, r_e)


def test_viscous_part_is_linear_in_mu():
    r = {mu: oracle.Oracle(P.ns_vortex_2d(4, 3, mu=mu)).compute_rhs(P.ns_vortex_2d(4, 3, mu=mu).sol)[0]
         for mu in (0.0, 0.01, 0.02)}
    v1, v2 = r[0.01] - r[0.0], r[0.02] - r[0.0]
    assert np.max(np.abs(v2 - 2.0 * v1)) <= 1e-11 * np.max(np.abs(v1))
    assert np.max(np.abs(v1)) > 1e-3


@pytest.mark.parametrize("mk", [lambda: P.ns_vortex_2d(4, 3), lambda: P.ns_taylor_green(3, 2, amplitude=0.1)])
def test_constant_state_is_steady(mk):
    prob = mk()
    vals = [1.0, 0.3, -0.2] + ([0.1] if prob.d == 3 else []) + [2.5]
    assert oracle.Oracle(prob).compute_rhs(P.constant_state(prob, vals))[1] < 1e-11


@pytest.mark.parametrize("mk", [lambda: P.ns_vortex_2d(4, 3, mu=0.05), lambda: P.ns_taylor_green(3, 2, Re=100.0)])
def test_conservation(mk):
    prob = mk()
    raw = oracle.Oracle(prob).compute_rhs_raw(prob.sol)
    tot = raw.sum(axis=(0, 2))
    assert np.all(np.abs(tot) <= 1e-12 * np.abs(raw).sum(axis=(0, 2)).max())


@pytest.mark.parametrize("mk", [lambda: P.ns_vortex_2d(3, 2, mu=0.05),
                                lambda: P.ns_taylor_green(2, 2, Re=50.0, viscosity=P.VISCOSITY_SUTHERLAND)])
def test_complex_step_matches_central_differences(mk):
    prob = mk()
    o = oracle.Oracle(prob)
    rng = np.random.default_rng(1)
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    dirn = rng.standard_normal(prob.sol.shape)
    _, ri = o.compute_rhs_cmplx(base, 1e-30 * dirn)
    jv = ri / 1e-30
    eps = 1e-6
    rp, _ = o.compute_rhs(base + eps * dirn)
    rm, _ = o.compute_rhs(base - eps * dirn)
    assert np.max(np.abs(jv - (rp - rm) / (2 * eps))) <= 1e-6 * np.max(np.abs(jv))


def test_sutherland_viscosity_differs_from_constant():
    rc, _ = oracle.Oracle(P.ns_vortex_2d(3, 2, mu=0.05)).compute_rhs(P.ns_vortex_2d(3, 2, mu=0.05).sol)
    ps = P.ns_vortex_2d(3, 2, mu=0.05, viscosity=P.VISCOSITY_SUTHERLAND)
    rs, _ = oracle.Oracle(ps).compute_rhs(ps.sol)
    assert np.max(np.abs(rs - rc)) > 1e-6


def _viscous_flux(U, dU, mu):
    """Viscous flux (2, 4, ...) of the 2D Navier-Stokes equations (the flux the residual subtracts)."""
    rho, E = U[0], U[3]
    u = U[1:3] / rho
    du = [[(dU[x][1 + s] - dU[x][0] * u[s]) / rho for x in range(2)] for s in range(2)]   # du[s][x]
    div = du[0][0] + du[1][1]
    tau = [[mu * 2 * (du[a][a] - div / 3) if a == b else mu * (du[b][a] + du[a][b]) for b in range(2)]
           for a in range(2)]
    F = np.zeros((2, 4) + rho.shape)
    for x in range(2):
        dTs = (dU[x][3] * rho - E * dU[x][0]) / rho ** 2 - sum(u[k] * du[k][x] for k in range(2))
        for k in range(2):
            F[x][1 + k] = tau[k][x]
        F[x][3] = P.GAMMA / PR * mu * dTs + sum(u[k] * tau[x][k] for k in range(2))
    return F


def _exact_viscous_divergence(X, Y, mu):
    def grad(X, Y, h=1e-4):
        f = P.ns_field_2d
        gx = (-f(X + 2 * h, Y) + 8 * f(X + h, Y) - 8 * f(X - h, Y) + f(X - 2 * h, Y)) / (12 * h)
        gy = (-f(X, Y + 2 * h) + 8 * f(X, Y + h) - 8 * f(X, Y - h) + f(X, Y - 2 * h)) / (12 * h)
        return np.stack([gx, gy])

    def FV(X, Y):
        return _viscous_flux(P.ns_field_2d(X, Y), grad(X, Y), mu)
    h = 1e-3
    return (FV(X + h, Y)[0] - FV(X - h, Y)[0]) / (2 * h) + (FV(X, Y + h)[1] - FV(X, Y - h)[1]) / (2 * h)


def test_viscous_operator_converges_to_the_divergence_of_the_viscous_flux():
    mu, p = 0.05, 3
    errs = []
    for n in (8, 16):
        r1, _ = oracle.Oracle(P.ns_periodic_field_2d(n, p, mu=mu)).compute_rhs(P.ns_periodic_field_2d(n, p, mu=mu).sol)
        p0 = P.ns_periodic_field_2d(n, p, mu=0.0)
        r0, _ = oracle.Oracle(p0).compute_rhs(p0.sol)
        x = p0.solution_node_xyz()
        exact = np.transpose(_exact_viscous_divergence(x[..., 0], x[..., 1], mu), (1, 0, 2))
        errs.append(np.max(np.abs(r1 - r0 - exact)))
    assert errs[1] < errs[0] / 3.5      # h^(p-1) = h^2 for p = 3 (observed ratio 4.65)


# ---- boundaries: no-slip adiabatic walls and the Euler boundary values with the interior gradient ----------------
def _at_rest(prob, p):
    return P.constant_state(prob, [1.0] + [0.0] * prob.d + [p / P.GM1])


@pytest.mark.parametrize("d,flux", [(2, P.NUM_FLUX_ROE_PIKE), (3, P.NUM_FLUX_LAX_FRIEDRICHS)])
def test_fluid_at_rest_between_no_slip_walls_is_steady(d, flux):
    prob = P.ns_channel(d, 3, 2, num_flux=flux, amplitude=0.05)
    assert oracle.Oracle(prob).compute_rhs(_at_rest(prob, 2.0))[1] < 1e-11


def test_no_slip_walls_conserve_mass():
    """Lax-Friedrichs with the mirrored momentum and no viscous mass flux: nothing crosses the walls."""
    prob = P.ns_channel(2, 4, 3, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS)
    raw = oracle.Oracle(prob).compute_rhs_raw(prob.sol)
    assert abs(raw[:, 0].sum()) <= 1e-13 * np.abs(raw[:, 0]).sum()


def test_adiabatic_walls_conserve_energy():
    """The wall's normal energy flux is set to zero, so total energy only moves between volumes."""
    prob = P.ns_channel(2, 4, 3, num_flux=P.NUM_FLUX_ROE_PIKE)
    raw = oracle.Oracle(prob).compute_rhs_raw(prob.sol)
    assert abs(raw[:, 3].sum()) <= 1e-12 * np.abs(raw[:, 3]).sum()


def test_riemann_boundaries_keep_the_free_stream():
    prob = P.ns_riemann_vortex_2d(4, 3)
    vals = [1.0, 1.0, 1.0, 1.0 / P.GM1 + 1.0]   # the exterior stream (1, 1, 1, 1)
    assert oracle.Oracle(prob).compute_rhs(P.constant_state(prob, vals))[1] < 1e-11


@pytest.mark.parametrize("mk", [lambda: P.ns_channel(2, 3, 2, mu=0.05), lambda: P.ns_riemann_vortex_2d(3, 2, mu=0.05),
                                lambda: P.ns_channel(3, 2, 2, mu=0.05)])
def test_boundary_complex_step(mk):
    prob = mk()
    o = oracle.Oracle(prob)
    rng = np.random.default_rng(4)
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    dirn = rng.standard_normal(prob.sol.shape)
    _, ri = o.compute_rhs_cmplx(base, 1e-30 * dirn)
    jv = ri / 1e-30
    eps = 1e-6
    rp, _ = o.compute_rhs(base + eps * dirn)
    rm, _ = o.compute_rhs(base - eps * dirn)
    assert np.max(np.abs(jv - (rp - rm) / (2 * eps))) <= 1e-6 * np.max(np.abs(jv))


def test_ns_refuses_euler_only_boundaries():
    prob = P.euler_channel_2d(3, 2)              # slip walls: an Euler boundary the reference's NS does not take
    prob.pde, prob.ns = P.PDE_NAVIER_STOKES, {"viscosity": 101, "mu": 0.01, "Pr": 0.72, "r_s": 1.0}
    with pytest.raises(Exception):
        oracle.Oracle(prob).compute_rhs(prob.sol)


# ---- the rotating and diabatic walls of the Taylor-Couette case ----------------------------------------------------
def test_taylor_couette_at_rest_is_steady():
    """omega = 0: the rotating wall's state (rho_b, 0, E_b) equals the interior's, the outer wall is adiabatic."""
    prob = P.ns_taylor_couette(4, 3, mu=0.02, omega=0.0)
    assert oracle.Oracle(prob).compute_rhs(_at_rest(prob, 1.0))[1] < 1e-11


def test_diabatic_wall_without_heat_flux_is_the_adiabatic_wall():
    pa = P.ns_taylor_couette(4, 3, mu=0.02, perturb=0.05)
    pd = P.ns_taylor_couette(4, 3, mu=0.02, perturb=0.05, diabatic=True, dTdn=0.0)
    assert np.array_equal(oracle.Oracle(pa).compute_rhs(pa.sol)[0], oracle.Oracle(pd).compute_rhs(pd.sol)[0])


def test_diabatic_wall_adds_its_heat_flux():
    """The wall's energy flux nf_E = -mu Cp / Pr dTdn replaces the computed one, so switching dTdn on (same state)
    adds mu Cp / Pr dTdn times the wall's length to the total energy, and nothing else changes. The length is the
    face quadrature of the curved wall (sum of w_f J_f), within 1e-6 of 2 pi r_o at 8 volumes around."""
    mu, dTdn = 0.02, 1.0
    p1 = P.ns_taylor_couette(8, 3, mu=mu, diabatic=True, dTdn=dTdn, perturb=0.05)
    p0 = P.ns_taylor_couette(8, 3, mu=mu, diabatic=True, dTdn=dTdn, perturb=0.05)
    p0.ns["dTdn"] = 0.0
    d = oracle.Oracle(p1).compute_rhs_raw(p1.sol) - oracle.Oracle(p0).compute_rhs_raw(p0.sol)
    q = mu * (P.GAMMA / P.GM1) / 0.72 * dTdn
    wall = p1.bc == P.BC_NOSLIP_DIABATIC
    length = float((p1.geom.jacobian_det_fc[wall] * p1.ops.w_fc[None, :]).sum())
    assert abs(length - 2.0 * np.pi) <= 1e-6 * 2.0 * np.pi
    assert abs(d[:, 3].sum() - q * length) <= 1e-12 * q * length
    assert np.max(np.abs(d[:, :3])) == 0.0


@pytest.mark.parametrize("diabatic", [False, True])
def test_taylor_couette_complex_step(diabatic):
    prob = P.ns_taylor_couette(3, 2, mu=0.05, diabatic=diabatic, perturb=0.05)
    o = oracle.Oracle(prob)
    rng = np.random.default_rng(5)
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    dirn = rng.standard_normal(prob.sol.shape)
    _, ri = o.compute_rhs_cmplx(base, 1e-30 * dirn)
    jv = ri / 1e-30
    eps = 1e-6
    rp, _ = o.compute_rhs(base + eps * dirn)
    rm, _ = o.compute_rhs(base - eps * dirn)
    assert np.max(np.abs(jv - (rp - rm) / (2 * eps))) <= 1e-6 * np.max(np.abs(jv))


def test_diabatic_heat_flux_needs_constant_viscosity():
    prob = P.ns_taylor_couette(3, 2, diabatic=True)
    prob.ns["viscosity"] = P.VISCOSITY_SUTHERLAND
    with pytest.raises(Exception):
        oracle.Oracle(prob).compute_rhs(prob.sol)
