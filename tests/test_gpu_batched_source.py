"""The source term in the batched context (dgpu_batch_set_source) against the oracle, through the C ABI.

The oracle adds tw0_vt_vc (J s) to every volume's rhs before M^-1 (compute_source_rhs_dg_like, compute_rlhs.c:47-57).
Cases: seeded sources on the mixed-order HEX mesh (TP groups: s at the GL nodes), on the mixed HEX/TET/WEDGE/PYR mesh
(dense groups: cv0^T diag(w J) s formed once on the host) and on the mixed-order Navier-Stokes channel. Residual
and SSP-RK3 states to 1e-12 normwise relative error in every launch form the case takes; removing the source gives
the source-free residual bit for bit; a source set after steps were captured reaches the next steps.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import mixed as M
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _with_source(prob, seed, scale=0.01):
    n_vc = np.array([int(g.n_vc) for g in prob.groups])[np.asarray(prob.vol_group)]
    rng = np.random.default_rng(seed)
    prob.source_vc = scale * rng.standard_normal(int(n_vc.sum()) * prob.n_var)
    return prob


def _types():
    from dpgsolver_gb300.host.mixed_types import mixed_types_euler
    return _with_source(mixed_types_euler(4, seed=1), 2)


CASES = {
    "hex_roe_mixed_4": (lambda: _with_source(M.mixed_euler(3, 4, seed=0), 1), ["plain", "fused", "branches", "stage"]),
    "types_roe_4": (_types, ["plain", "fused", "branches", "stage"]),
    "ns_quad_walls_5": (lambda: _with_source(M.mixed_ns(2, 5, seed=3, walls={(1, 0): P.BC_NOSLIP_ADIABATIC,
                                                                            (1, 1): P.BC_RIEMANN}), 3),
                        ["plain", "branches"]),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_batched_source_matches_oracle(gpu_lib, name):
    from dpgsolver_gb300.solver import BatchSimulation
    make, forms = CASES[name]
    prob = make()
    o = oracle.Oracle(prob)
    r_ref, mx_ref = o.compute_rhs(prob.sol)
    s_ref = prob.sol.copy()
    for _ in range(2):
        s_ref, _, _ = o.ssp_rk3_step(s_ref, prob.dt)
    with BatchSimulation(prob) as sim:
        for form in forms:
            sim.form = form
            sim.upload_state(prob.sol)
            mx = sim.compute_rhs()
            assert _rel(sim.rhs, r_ref) <= TOL, form
            assert abs(mx - mx_ref) <= TOL * mx_ref
            sim.upload_state(prob.sol)
            sim.ssp_rk3_steps(prob.dt, 2)
            assert _rel(sim.sol_coef, s_ref) <= TOL, form


def test_removing_and_setting_the_source_after_capture(gpu_lib):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES["hex_roe_mixed_4"][0]()
    src = prob.source_vc
    prob.source_vc = None
    with BatchSimulation(prob) as plain:
        plain.compute_rhs()
        r_plain = plain.rhs
    prob.source_vc = src
    o = oracle.Oracle(prob)
    s_ref = prob.sol.copy()
    for _ in range(2):
        s_ref, _, _ = o.ssp_rk3_step(s_ref, prob.dt)
    with BatchSimulation(prob) as sim:
        sim.set_source(None)
        sim.compute_rhs()
        assert np.array_equal(sim.rhs, r_plain)
        sim.ssp_rk3_steps(prob.dt, 2)          # the steps are captured without a source
        sim.set_source(src)
        sim.upload_state(prob.sol)
        sim.ssp_rk3_steps(prob.dt, 2)
        assert _rel(sim.sol_coef, s_ref) <= TOL
        with pytest.raises(ValueError):
            sim.set_source(src[:-1])
