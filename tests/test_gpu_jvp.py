"""Forward-mode linearisation (dgpu_jvp) against the oracle's complex step, the reference's own linearisation
(compute_lhs_cmplx_step_dg, test_support_solve_dg.c:83-110), and against the adjoint (dgpu_vjp_backward).

Both the dual-number product and complex step (h = 1e-30) are exact to rounding, so the bar is the residual's:
<= 1e-12 normwise relative. States are perturbed additively by 1e-2 so that no face node sits on a kink of the
numerical fluxes (equal traces, Vn = 0), where the two linearisations may take different one-sided branches.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12

CASES = {
    "adv2d_p2_8": lambda: P.advection_2d(8, 2),
    "vortex2d_roe_p3_6": lambda: P.euler_vortex_2d(6, 3),
    "vortex2d_lf_p2_6": lambda: P.euler_vortex_2d(6, 2, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "hex_lf_p3_4": lambda: P.euler_hex_3d(4, 3),
    "hex_roe_p2_4": lambda: P.euler_hex_3d(4, 2, num_flux=P.NUM_FLUX_ROE_PIKE),
    "hex_roe_p4_2": lambda: P.euler_hex_3d(2, 4, num_flux=P.NUM_FLUX_ROE_PIKE),
}


def rel_err(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _inputs(prob, seed):
    rng = np.random.default_rng(seed)
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    return base, rng.standard_normal(prob.sol.shape)


@pytest.mark.parametrize("name", sorted(CASES))
def test_jvp_matches_complex_step(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    base, dirn = _inputs(prob, 7)
    o = oracle.Oracle(prob)
    r_ref, ri = o.compute_rhs_cmplx(base, 1e-30 * dirn)
    jv_ref = ri / 1e-30
    with Simulation(prob) as sim:
        r, jv = sim.jvp(base, dirn)
    assert rel_err(r, r_ref) <= TOL
    assert rel_err(jv, jv_ref) <= TOL


@pytest.mark.parametrize("name", ["vortex2d_roe_p3_6", "hex_roe_p2_4"])
def test_jvp_is_the_adjoint_of_the_vjp(gpu_lib, name):
    """<v, J d> = <J^T v, d> for seeded v, d: the forward and reverse linearisations are transposes."""
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    base, dirn = _inputs(prob, 11)
    v = np.random.default_rng(12).standard_normal(prob.sol.shape)
    with Simulation(prob) as sim:
        _, jv = sim.jvp(base, dirn)
        sim.vjp_forward(base)
        g = sim.vjp_backward(v)
    lhs, rhs = float(np.sum(v * jv)), float(np.sum(g * dirn))
    assert abs(lhs - rhs) <= 1e-12 * np.sqrt(np.sum(v * v) * np.sum(jv * jv))


def test_jvp_is_linear_in_the_direction(gpu_lib):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES["hex_lf_p3_4"]()
    base, d1 = _inputs(prob, 3)
    d2 = np.random.default_rng(4).standard_normal(prob.sol.shape)
    with Simulation(prob) as sim:
        _, j1 = sim.jvp(base, d1)
        _, j2 = sim.jvp(base, d2)
        _, j12 = sim.jvp(base, 2.0 * d1 - 0.5 * d2)
    assert rel_err(j12, 2.0 * j1 - 0.5 * j2) <= 1e-13
