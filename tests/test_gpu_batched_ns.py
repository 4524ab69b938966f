"""Navier-Stokes in the batched mixed-order context, through the C ABI, against the oracle.

The oracle restates the reference's BR2 data flow with dense operators per volume and face operators at each face's
order p_f = max(p_L, p_R); it is pinned to the reference's own Navier-Stokes outputs on uniform meshes and to its
mixed-order faces on Euler and advection. Here: QUAD and HEX meshes with p in {1, 2, 3, 4} per volume (seeded),
periodic or with no-slip adiabatic / diabatic / rotating walls and Riemann faces, straight and curved, Roe-Pike and
Lax-Friedrichs, constant and Sutherland viscosity. Residual and SSP-RK3 states to 1e-12 normwise relative error, in
both launch forms that take Navier-Stokes (per-group launches, and the same on parallel graph branches), which agree
bit for bit; the persistent forms refuse it.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import mixed as M
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12

CASES = {
    "quad_roe_periodic_6": lambda: M.mixed_ns(2, 6, seed=1),
    "quad_lf_suth_periodic_5": lambda: M.mixed_ns(2, 5, seed=2, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS,
                                                  viscosity=P.VISCOSITY_SUTHERLAND, mu=0.05),
    "quad_roe_walls_6": lambda: M.mixed_ns(2, 6, seed=3, walls={(1, 0): P.BC_NOSLIP_ADIABATIC,
                                                                (1, 1): P.BC_NOSLIP_ALL_ROTATING}),
    "quad_lf_diabatic_riemann_curved_5": lambda: M.mixed_ns(2, 5, seed=4, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS,
                                                            curved=True, dTdn=0.5,
                                                            walls={(1, 0): P.BC_NOSLIP_DIABATIC,
                                                                   (1, 1): P.BC_RIEMANN}),
    "hex_roe_periodic_curved_3": lambda: M.mixed_ns(3, 3, seed=5, curved=True),
    "hex_lf_walls_3": lambda: M.mixed_ns(3, 3, seed=6, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS,
                                         walls={(1, 0): P.BC_NOSLIP_ADIABATIC, (1, 1): P.BC_NOSLIP_ADIABATIC}),
}


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("form", ["plain", "branches"])
def test_ns_residual_and_rk3_match_oracle(gpu_lib, name, form):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES[name]()
    assert len(set(int(p) for p in prob.p_vol)) > 1
    o = oracle.Oracle(prob)
    r_ref, mx_ref = o.compute_rhs(prob.sol)
    s_ref = prob.sol.copy()
    for _ in range(3):
        s_ref, mx_s, _ = o.ssp_rk3_step(s_ref, prob.dt)
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx = sim.compute_rhs()
        assert _rel(sim.rhs, r_ref) <= TOL
        assert abs(mx - mx_ref) <= TOL * mx_ref
        mx = sim.ssp_rk3_steps(prob.dt, 3)
        assert _rel(sim.sol_coef, s_ref) <= TOL
        assert abs(mx - mx_s) <= 1e-10 * mx_s


def test_ns_forms_agree_bitwise_and_persistent_forms_refuse(gpu_lib):
    from dpgsolver_gb300._lib import DGPUError
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES["hex_lf_walls_3"]()
    out = []
    with BatchSimulation(prob) as sim:
        for form in ("plain", "branches"):
            sim.form = form
            sim.upload_state(prob.sol)
            sim.compute_rhs()
            r = sim.rhs
            sim.ssp_rk3_steps(prob.dt, 2, want_max=False)
            out.append((r, sim.sol_coef))
        for form in ("fused", "stage"):
            with pytest.raises(DGPUError):
                sim.form = form
        rep = sim.autotune(prob.dt, reps=1)
        assert "plain" in rep and "branches" in rep
        assert sim.form in ("plain", "branches")
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_ns_single_order_mesh_matches_oracle(gpu_lib):
    """One group (every volume at p = 3): no interpolation between orders, walls and a Riemann side."""
    from dpgsolver_gb300.solver import BatchSimulation
    prob = M.mixed_ns(2, 5, p_set=(3,), seed=7, walls={(1, 0): P.BC_NOSLIP_ADIABATIC, (1, 1): P.BC_RIEMANN})
    r_ref, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    with BatchSimulation(prob) as sim:
        sim.compute_rhs()
        assert _rel(sim.rhs, r_ref) <= TOL


def test_ns_with_dense_groups_is_refused(gpu_lib):
    """TRI/TET/WEDGE/PYR groups have no Navier-Stokes path in the batched context: DGPU_ERR_UNSUPPORTED."""
    from dpgsolver_gb300._lib import DGPUError
    from dpgsolver_gb300.host.mixed_types import mixed_tri_quad_euler
    from dpgsolver_gb300.solver import BatchSimulation
    prob = mixed_tri_quad_euler(4, seed=0)
    prob.pde, prob.ns = P.PDE_NAVIER_STOKES, {"viscosity": 101, "mu": 0.01, "Pr": 0.72, "r_s": 1.0}
    with pytest.raises(DGPUError) as e:
        BatchSimulation(prob)
    assert e.value.status == 2
