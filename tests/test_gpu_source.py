"""The source term on the GPU (dgpu_set_source) against the oracle, through the C ABI.

Cases: the reference's steady advection case (s = b . grad u) on the periodic and the non-periodic curved box, and
seeded random sources on the curved HEX Euler vortex and the Navier-Stokes vortex. Residual and SSP-RK3 states to
1e-12 normwise relative error. Also: removing the source gives back the source-free residual bit for bit; a source
set after steps were captured reaches the next steps; the linearisations' primal includes the source while their
derivative is the source-free one; a source of the wrong shape is refused on the host.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _random_source(prob, seed, scale=0.01):
    rng = np.random.default_rng(seed)
    mag = np.abs(prob.sol).max(axis=(0, 2), keepdims=True)
    return scale * mag * rng.standard_normal(prob.sol.shape)


def _hex():
    prob = P.euler_hex_3d(3, 2)
    prob.source_vc = _random_source(prob, 1)
    return prob


def _ns():
    prob = P.ns_vortex_2d(4, 3)
    prob.source_vc = _random_source(prob, 2)
    return prob


CASES = {
    "adv_default_p3_8": lambda: P.advection_default_2d(8, 3),
    "adv_default_bc_p2_6": lambda: P.advection_default_2d(6, 2, periodic=False),
    "hex_lf_p2_3": _hex,
    "ns_vortex_p3_4": _ns,
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_residual_and_rk3_with_source_match_oracle(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    o = oracle.Oracle(prob)
    r_ref, mx_ref = o.compute_rhs(prob.sol)
    s_ref = prob.sol
    for _ in range(5):
        s_ref, _, _ = o.ssp_rk3_step(s_ref, prob.dt)
    with Simulation(prob) as sim:
        mx = sim.compute_rhs()
        assert _rel(sim.rhs, r_ref) <= TOL
        assert abs(mx - mx_ref) <= TOL * mx_ref
        sim.upload_state(prob.sol)
        sim.ssp_rk3_steps(prob.dt, 5)
        assert _rel(sim.sol_coef, s_ref) <= TOL


def test_removing_the_source_and_setting_it_after_capture(gpu_lib):
    from dpgsolver_gb300.solver import Simulation
    prob = P.advection_default_2d(6, 3, periodic=False)
    src = prob.source_vc
    prob.source_vc = None
    with Simulation(prob) as plain:
        plain.compute_rhs()
        r_plain = plain.rhs
    prob.source_vc = src
    o = oracle.Oracle(prob)
    s_ref = prob.sol
    for _ in range(3):
        s_ref, _, _ = o.ssp_rk3_step(s_ref, prob.dt)
    with Simulation(prob) as sim:
        sim.set_source(None)
        sim.compute_rhs()
        assert np.array_equal(sim.rhs, r_plain)
        sim.ssp_rk3_steps(prob.dt, 3)          # the steps are captured without a source
        sim.set_source(src)
        sim.upload_state(prob.sol)
        sim.ssp_rk3_steps(prob.dt, 3)
        assert _rel(sim.sol_coef, s_ref) <= TOL
        with pytest.raises(ValueError):
            sim.set_source(src[:, :, :-1])


def test_linearisation_primal_includes_the_source(gpu_lib):
    from dpgsolver_gb300.solver import Simulation
    prob = _hex()
    d = np.random.default_rng(3).standard_normal(prob.sol.shape)
    r_ref, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    src = prob.source_vc
    prob.source_vc = None
    with Simulation(prob) as plain:
        _, jv_plain = plain.jvp(prob.sol, d)
    prob.source_vc = src
    with Simulation(prob) as sim:
        r, jv = sim.jvp(prob.sol, d)
        assert _rel(r, r_ref) <= TOL
        assert np.array_equal(jv, jv_plain)
        r2, _ = sim.vjp_forward(prob.sol)
        assert _rel(r2, r_ref) <= TOL
