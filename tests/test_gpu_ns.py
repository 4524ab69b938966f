"""Navier-Stokes on the CUDA path (Euler flux + viscous flux with BR2 gradients in GL nodal space) against the
oracle's restatement of the reference's data flow (compute_grad_coef_dg_T, constructor_partial_grad_fc_interp,
the central viscous numerical flux), at <= 1e-12 normwise relative as in test_gpu_parity.py.

On the Taylor-Green vortex the residual (0.5 to 3 here, smaller the finer the mesh) is what remains after terms
of the size of the background pressure 1 / (gamma Ma^2) (7.9 at Mach 0.3, 71 at Mach 0.1) cancel, so its rounding
noise relative to max|R| is far above the other cases': the oracle's own response to one-ulp perturbations of its
input (the noise floor, measured per case) reaches 1.2e-11 on 12^3 p = 3; the Mach 0.3 channel (background
pressure 7.9) sits at 1e-12. Every residual case is therefore held to max(1e-12, 4 x its measured floor): where the
floor is low (the vortex cases, below 3e-13) the plain bound is the one that applies.

The Taylor-Couette cases (the reference's navier_stokes/steady/taylor_couette on a curved annulus) cover the
rotating wall (BC_NOSLIP_ALL_ROTATING: 2 s_wall - s_l) and the diabatic wall (BC_NOSLIP_DIABATIC: the energy flux
-mu Cp / Pr dTdn). Their volumes are stretched (aspect ratio up to 12) and the oracle's noise floor there is about
7e-12, so the same max(1e-12, 4 x floor) rule applies.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300 import _lib
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12

CASES = {
    "vortex2d_roe_p3_8": lambda: P.ns_vortex_2d(8, 3, mu=0.01),
    "vortex2d_lf_p2_6": lambda: P.ns_vortex_2d(6, 2, mu=0.05, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "vortex2d_suth_p4_4": lambda: P.ns_vortex_2d(4, 4, mu=0.05, viscosity=P.VISCOSITY_SUTHERLAND),
    "field2d_p3_8": lambda: P.ns_periodic_field_2d(8, 3, mu=0.05),
    "tgv_p3_4_curved": lambda: P.ns_taylor_green(4, 3, Re=100.0, mach=0.3, amplitude=0.1),
    "tgv_p2_6": lambda: P.ns_taylor_green(6, 2, Re=400.0, mach=0.3),
    "tgv_p4_2_lf": lambda: P.ns_taylor_green(2, 4, Re=50.0, mach=0.3, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "tgv_p1_4_suth": lambda: P.ns_taylor_green(4, 1, Re=200.0, mach=0.3, viscosity=P.VISCOSITY_SUTHERLAND),
    # many CTAs
    "tgv_p3_12": lambda: P.ns_taylor_green(12, 3, Re=1600.0, mach=0.3),
    # boundaries: no-slip adiabatic walls, Riemann sides
    "channel2d_roe_p3_6": lambda: P.ns_channel(2, 6, 3, mu=0.02, amplitude=0.05),
    "channel3d_lf_p2_4": lambda: P.ns_channel(3, 4, 2, mu=0.02, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "channel3d_roe_p3_4": lambda: P.ns_channel(3, 4, 3, mu=0.01, amplitude=0.05),
    "riemann2d_roe_p3_6": lambda: P.ns_riemann_vortex_2d(6, 3, mu=0.02),
    # the Taylor-Couette annulus: rotating inner wall, adiabatic or diabatic outer wall
    "couette_roe_p3_6": lambda: P.ns_taylor_couette(6, 3, mu=0.02, perturb=0.2),
    "couette_diab_lf_p2_8": lambda: P.ns_taylor_couette(8, 2, mu=0.02, diabatic=True, perturb=0.2,
                                                         num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "couette_diab_roe_p4_4": lambda: P.ns_taylor_couette(4, 4, mu=0.01, diabatic=True, perturb=0.2),
}


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def noise_floor(o, sol, r_ref, seeds=3):
    """max over seeds of rel(R(sol (1 +- 2^-52)), R(sol)): the oracle's response to one-ulp input noise."""
    out = 0.0
    for seed in range(seeds):
        noisy = sol * (1.0 + np.random.default_rng(seed).choice([-1.0, 1.0], sol.shape) * 2.0 ** -52)
        out = max(out, rel(o.compute_rhs(noisy)[0], r_ref))
    return out


@pytest.mark.parametrize("name", sorted(CASES))
def test_ns_residual_matches_oracle(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    o = oracle.Oracle(prob)
    r_ref, mx_ref = o.compute_rhs(prob.sol)
    tol = max(TOL, 4.0 * noise_floor(o, prob.sol, r_ref))
    with Simulation(prob) as sim:
        mx = sim.compute_rhs()
        r = sim.rhs
    assert rel(r, r_ref) <= tol
    assert abs(mx - mx_ref) <= tol * mx_ref


def test_ns_mach01_taylor_green_within_the_oracle_noise_floor(gpu_lib):
    from dpgsolver_gb300.solver import Simulation
    prob = P.ns_taylor_green(6, 2, Re=1600.0, mach=0.1)
    o = oracle.Oracle(prob)
    r_ref, _ = o.compute_rhs(prob.sol)
    floor = noise_floor(o, prob.sol, r_ref)
    with Simulation(prob) as sim:
        sim.compute_rhs()
        r = sim.rhs
    assert rel(r, r_ref) <= 4.0 * floor


@pytest.mark.parametrize("name", ["vortex2d_roe_p3_8", "tgv_p3_4_curved", "tgv_p2_6", "channel3d_roe_p3_4",
                                  "riemann2d_roe_p3_6", "couette_diab_lf_p2_8"])
def test_ns_rk3_steps_match_oracle(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    ref = oracle.Oracle(prob)
    s_ref = prob.sol.copy()
    for _ in range(4):
        s_ref, mx_ref, _ = ref.ssp_rk3_step(s_ref, prob.dt)
    with Simulation(prob) as sim:
        mx = sim.ssp_rk3_steps(prob.dt, 4)
        s = sim.sol_coef
    assert rel(s, s_ref) <= TOL   # the state itself is O(1): no cancellation
    assert abs(mx - mx_ref) <= 1e-10 * mx_ref


def test_ns_zero_viscosity_is_the_euler_path(gpu_lib):
    """mu = 0: the four-kernel Navier-Stokes stage gives the three-kernel Euler stage's residual (the two are
    compiled separately, so they may differ by rounding: held to the oracle's noise floor of the Euler case)."""
    from dpgsolver_gb300.solver import Simulation
    pn, pe = P.ns_vortex_2d(8, 3, mu=0.0), P.euler_vortex_2d(8, 3)
    with Simulation(pn) as a, Simulation(pe) as b:
        a.compute_rhs()
        b.compute_rhs()
        ra, rb = a.rhs, b.rhs
    o = oracle.Oracle(pe)
    r_ref, _ = o.compute_rhs(pe.sol)
    assert rel(ra, rb) <= max(TOL, 4.0 * noise_floor(o, pe.sol, r_ref))


def test_ns_free_stream(gpu_lib):
    from dpgsolver_gb300.solver import Simulation
    for prob in (P.ns_vortex_2d(8, 3), P.ns_taylor_green(4, 3, amplitude=0.1)):
        vals = [1.0, 0.3, -0.2] + ([0.1] if prob.d == 3 else []) + [2.5]
        with Simulation(prob) as sim:
            sim.upload_state(P.constant_state(prob, vals))
            assert sim.compute_rhs() < 1e-11
    # fluid at rest between no-slip walls; the exterior stream inside Riemann sides
    for prob, vals in ((P.ns_channel(3, 4, 3, amplitude=0.05), [1.0, 0.0, 0.0, 0.0, 2.0 / P.GM1]),
                       (P.ns_riemann_vortex_2d(6, 3), [1.0, 1.0, 1.0, 1.0 / P.GM1 + 1.0]),
                       (P.ns_taylor_couette(6, 3, omega=0.0), [1.0, 0.0, 0.0, 1.0 / P.GM1])):
        with Simulation(prob) as sim:
            sim.upload_state(P.constant_state(prob, vals))
            assert sim.compute_rhs() < 1e-11


# ---- forward-mode linearisation and the block-sparse Jacobian ------------------------------------------------------
JVP_CASES = ["vortex2d_roe_p3_8", "vortex2d_lf_p2_6", "vortex2d_suth_p4_4", "tgv_p3_4_curved", "tgv_p1_4_suth",
             "tgv_p4_2_lf", "channel2d_roe_p3_6", "channel3d_lf_p2_4", "riemann2d_roe_p3_6", "couette_roe_p3_6",
             "couette_diab_lf_p2_8"]


def _inputs(prob, seed):
    rng = np.random.default_rng(seed)
    return prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape), rng.standard_normal(prob.sol.shape)


def jvp_noise_floor(o, base, dirn, jv_ref, seeds=3):
    """The oracle's complex-step J d response to one-ulp noise in the state (as noise_floor for the residual)."""
    out = 0.0
    for seed in range(seeds):
        noisy = base * (1.0 + np.random.default_rng(seed).choice([-1.0, 1.0], base.shape) * 2.0 ** -52)
        out = max(out, rel(o.compute_rhs_cmplx(noisy, 1e-30 * dirn)[1] / 1e-30, jv_ref))
    return out


@pytest.mark.parametrize("name", JVP_CASES)
def test_ns_jvp_matches_complex_step(gpu_lib, name):
    """dgpu_jvp on dual numbers against the oracle's complex step (h = 1e-30), both exact to rounding: the residual
    and J d at max(1e-12, 4 x the oracle's noise floor for each)."""
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    base, dirn = _inputs(prob, 7)
    o = oracle.Oracle(prob)
    r_ref, ri = o.compute_rhs_cmplx(base, 1e-30 * dirn)
    jv_ref = ri / 1e-30
    with Simulation(prob) as sim:
        r, jv = sim.jvp(base, dirn)
    assert rel(r, r_ref) <= max(TOL, 4.0 * noise_floor(o, base, r_ref))
    assert rel(jv, jv_ref) <= max(TOL, 4.0 * jvp_noise_floor(o, base, dirn, jv_ref))


def test_ns_jvp_is_linear_in_the_direction(gpu_lib):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES["channel2d_roe_p3_6"]()
    base, d1 = _inputs(prob, 3)
    d2 = np.random.default_rng(4).standard_normal(prob.sol.shape)
    with Simulation(prob) as sim:
        _, j1 = sim.jvp(base, d1)
        _, j2 = sim.jvp(base, d2)
        _, j12 = sim.jvp(base, 2.0 * d1 - 0.5 * d2)
    assert rel(j12, 2.0 * j1 - 0.5 * j2) <= 1e-13


JAC_CASES = {
    "vortex2d_roe_p2_3": lambda: P.ns_vortex_2d(3, 2, mu=0.05),
    "vortex2d_suth_lf_p1_4": lambda: P.ns_vortex_2d(4, 1, mu=0.05, viscosity=P.VISCOSITY_SUTHERLAND,
                                                    num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "tgv_p1_2": lambda: P.ns_taylor_green(2, 1, Re=50.0, mach=0.3, amplitude=0.1),
    "tgv_p2_2_suth": lambda: P.ns_taylor_green(2, 2, Re=50.0, mach=0.3, viscosity=P.VISCOSITY_SUTHERLAND),
    "channel2d_roe_p2_3": lambda: P.ns_channel(2, 3, 2, mu=0.05, amplitude=0.05),
    "channel3d_lf_p1_2": lambda: P.ns_channel(3, 2, 1, mu=0.05, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "riemann2d_roe_p2_3": lambda: P.ns_riemann_vortex_2d(3, 2, mu=0.05),
    "couette_roe_p2_3": lambda: P.ns_taylor_couette(3, 2, mu=0.05, perturb=0.05),
    "couette_diab_lf_p1_4": lambda: P.ns_taylor_couette(4, 1, mu=0.05, diabatic=True, perturb=0.05,
                                                         num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
}


@pytest.mark.parametrize("name", sorted(JAC_CASES))
def test_ns_jacobian_matches_complex_step(gpu_lib, name):
    """The BR2 residual of a volume depends on its face neighbours only (each face's lifting uses the two traces of
    that face), so the Euler block structure and distance-2 colouring carry over: the explicit and raw Jacobians
    against the oracle's complex-step Jacobian, column by column, at 1e-12 of max |J|."""
    from dpgsolver_gb300.solver import Simulation
    from test_gpu_jacobian import _complex_step_jacobian, _dense, _mass_rows
    prob = JAC_CASES[name]()
    base, _ = _inputs(prob, 3)
    J_cs, o = _complex_step_jacobian(prob, base)
    with Simulation(prob) as sim:
        nb, nnz, n_col = sim.jacobian_structure()
        rp, ci, vals = sim.jacobian(base, raw=False)
        _, _, vals_raw = sim.jacobian(base, raw=True)
    A = _dense(rp, ci, vals, nb)
    assert np.max(np.abs(A - J_cs)) <= TOL * np.max(np.abs(J_cs))
    J_raw = _mass_rows(prob, o, J_cs)
    assert np.max(np.abs(_dense(rp, ci, vals_raw, nb) - J_raw)) <= TOL * np.max(np.abs(J_raw))


def test_ns_refusals(gpu_lib):
    from dpgsolver_gb300.solver import BatchSimulation, Simulation
    prob = P.ns_taylor_couette(3, 2, mu=0.02, perturb=0.2)
    with Simulation(prob) as a, BatchSimulation(prob) as b:   # the batched context takes it as one group
        a.compute_rhs()
        b.compute_rhs()
        assert np.max(np.abs(b.rhs - a.rhs)) <= 1e-12 * np.max(np.abs(a.rhs))
    slip = P.euler_channel_2d(4, 2)             # slip walls: an Euler boundary the reference's NS does not take
    slip.pde, slip.ns = P.PDE_NAVIER_STOKES, {"viscosity": 101, "mu": 0.01, "Pr": 0.72, "r_s": 1.0}
    for ctx in (Simulation, BatchSimulation):
        with pytest.raises(_lib.DGPUError) as e:
            ctx(slip)
        assert e.value.status == 2
    bad = P.ns_vortex_2d(4, 2)
    bad.ns["Pr"] = 0.0
    with pytest.raises(_lib.DGPUError) as e:
        Simulation(bad)
    assert e.value.status == 1
    hot = P.ns_taylor_couette(3, 2, diabatic=True)   # a wall heat flux with Sutherland's law: the reference asserts
    hot.ns["viscosity"] = P.VISCOSITY_SUTHERLAND
    with pytest.raises(_lib.DGPUError) as e:
        Simulation(hot)
    assert e.value.status == 2
