"""Steady-state convergence of the GPU path on the reference's Euler supersonic vortex: the check the reference's own
integration tests run on this case (test_integration_convergence.c with its supersonic-vortex control files).

SSP-RK3 steps (graph-replayed, positivity limiter on) drive the state to a steady one (max |rhs| < 1e-9) on the
reference's parametric quarter annulus: curved volumes, Riemann faces with the exact solution outside, slip walls on
both arcs. The L2 error of the density against the exact solution must then fall at order p + 1 under refinement:
at least 2.7 for p = 2 (2 x 2, 4 x 4 and 8 x 8 volumes per block) and 3.0 for p = 3 (2 x 2, 4 x 4). p = 3 stays
below 4 on these meshes, as for the reference's isoparametric geometry (its own runs of this case use a
superparametric one for the optimal rate). The steady states on the coarse meshes match the oracle's.
"""
import os

import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import gmsh as G
from dpgsolver_gb300.host import problem as P
from dpgsolver_gb300.host.element import kron_tp
from dpgsolver_gb300.host.geometry import apply_nodes

pytestmark = pytest.mark.gpu
CFL_SCALE = 3.0      # dt = 3 x the problem's CFL-0.1 estimate (CFL 0.3, inside SSP-RK3's DG bound for p <= 3)
STEADY = 1e-9


def _density_error(prob, sol):
    ops, g = prob.ops, prob.geom
    rho = apply_nodes(kron_tp([ops.cv0_1d] * 2), np.ascontiguousarray(sol[:, 0, :])[..., None])[..., 0]
    exact = P.supersonic_vortex_state(g.xyz_vc[..., 0], g.xyz_vc[..., 1])[0]
    wJ = np.kron(ops.w_vc_1d, ops.w_vc_1d)[None, :] * g.jacobian_det_vc
    return float(np.sqrt(np.sum(wJ * (rho - exact) ** 2) / np.sum(wJ)))


def _steady_gpu(prob, max_steps=60000):
    from dpgsolver_gb300.solver import Simulation
    dt = CFL_SCALE * prob.dt
    with Simulation(prob) as sim:
        steps, mx = 0, np.inf
        while steps < max_steps and mx >= STEADY:
            mx = sim.ssp_rk3_steps(dt, 200)
            steps += 200
        return sim.sol_coef, mx, steps


def _steady_oracle(prob, max_steps=60000):
    o = oracle.Oracle(prob)
    s, dt, steps, mx = prob.sol.copy(), CFL_SCALE * prob.dt, 0, np.inf
    while steps < max_steps and mx >= STEADY:
        for _ in range(200):
            s, mx, _ = o.ssp_rk3_step(s, dt)
        steps += 200
    return s, mx, steps


@pytest.mark.parametrize("p,ns,rate", [(2, (2, 4, 8), 2.7), (3, (2, 4), 3.0)])
def test_supersonic_vortex_converges_at_order_p_plus_1(gpu_lib, tmp_path, p, ns, rate):
    errors = []
    for n in ns:
        path = str(tmp_path / f"sv_{n}.msh")
        G.write_quarter_square_annulus_msh(path, n, n)
        prob = P.euler_supersonic_vortex(path, p)
        sol, mx, steps = _steady_gpu(prob)
        assert mx < STEADY, (n, mx, steps)
        errors.append(_density_error(prob, sol))
        if n == ns[0]:   # the GPU's steady state is the oracle's
            sol_o, mx_o, _ = _steady_oracle(prob)
            assert mx_o < STEADY
            assert np.max(np.abs(sol - sol_o)) <= 1e-8 * np.max(np.abs(sol_o))
    rates = [float(np.log2(errors[k] / errors[k + 1])) for k in range(len(errors) - 1)]
    assert min(rates) >= rate, (errors, rates)
