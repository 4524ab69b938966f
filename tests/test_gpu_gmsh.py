"""The CUDA path on meshes read from gmsh files (dgpu_gmsh_read, include/dgpu_mesh.h) against the oracle.

The volumes of these meshes have random local frames and perturbed interior vertices, so neighbours see their
common faces in every orientation the reference distinguishes (the right traces are gathered through the face
permutations) and the straight volumes are not affine. Residual and SSP-RK3 steps at <= 1e-12 normwise relative,
as in test_gpu_parity.py; the context built from the volumes' vertices (device geometry) gives the same residual.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import gmsh as G
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _state(x):
    d = x.shape[1]
    rho = 1.0 + 0.2 * np.sin(0.7 * x[:, 0] + 0.3) * np.cos(0.5 * x[:, 1])
    vel = [0.5 + 0.1 * np.cos(0.4 * x[:, 1]), 0.3 + 0.1 * np.sin(0.6 * x[:, 0])]
    if d == 3:
        vel.append(0.2 + 0.05 * np.sin(0.3 * x[:, 2]))
    p = 1.0 + 0.1 * np.cos(0.3 * x[:, 0] + 0.2 * x[:, 1])
    return np.stack([rho] + [rho * v for v in vel] + [p / P.GM1 + 0.5 * rho * sum(v * v for v in vel)], axis=1)


def _adv_state(x):
    return (np.sin(0.5 * x[:, 0]) * np.cos(0.3 * x[:, 1]))[:, None]


CASES = {
    "hex_roe_p3_4_periodic": (3, 4, 3, P.NUM_FLUX_ROE_PIKE, True, None),
    "hex_lf_p2_6_periodic": (3, 6, 2, P.NUM_FLUX_LAX_FRIEDRICHS, True, None),
    "hex_roe_p2_4_bounded": (3, 4, 2, P.NUM_FLUX_ROE_PIKE, (False, True, False),
                             {(0, 0): 10101, (0, 1): 10101, (2, 0): 10102, (2, 1): 10102}),
    "quad_roe_p3_8_periodic": (2, 8, 3, P.NUM_FLUX_ROE_PIKE, True, None),
    "quad_lf_p4_6_bounded": (2, 6, 4, P.NUM_FLUX_LAX_FRIEDRICHS, (True, False), {(1, 0): 10102, (1, 1): 10101}),
}


def _problem(tmp_path, name, seed=11):
    d, n, p, flux, periodic, codes = CASES[name]
    path = tmp_path / f"{name}.msh"
    G.write_box_msh(path, d, n, 0.0, 10.0, periodic=periodic, codes=codes, rotate_seed=seed, perturb=0.2,
                    perturb_seed=4)
    return G.gmsh_tp_problem(path, d, p, P.PDE_EULER, flux, _state, exterior=_state)


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", sorted(CASES))
def test_gmsh_residual_and_steps_match_oracle(gpu_lib, tmp_path, name):
    from dpgsolver_gb300.solver import Simulation
    prob = _problem(tmp_path, name)
    o = oracle.Oracle(prob)
    r_ref, mx_ref = o.compute_rhs(prob.sol)
    s_ref = prob.sol.copy()
    for _ in range(3):
        s_ref, _, _ = o.ssp_rk3_step(s_ref, prob.dt)
    with Simulation(prob) as sim, Simulation(prob, device_geometry=True) as dev:
        mx = sim.compute_rhs()
        r = sim.rhs
        dev.compute_rhs()
        r_dev = dev.rhs
        sim.ssp_rk3_steps(prob.dt, 3)
        s = sim.sol_coef
    assert rel(r, r_ref) <= TOL
    assert abs(mx - mx_ref) <= TOL * mx_ref
    assert rel(r_dev, r_ref) <= TOL
    assert rel(s, s_ref) <= TOL


def test_gmsh_advection_upwind_box(gpu_lib, tmp_path):
    from dpgsolver_gb300.solver import Simulation
    path = tmp_path / "adv.msh"
    G.write_box_msh(path, 2, 6, 0.0, 10.0, periodic=False,
                    codes={(0, 0): 10041, (0, 1): 10041, (1, 0): 10041, (1, 1): 10041}, rotate_seed=2, perturb=0.2)
    prob = G.gmsh_tp_problem(path, 2, 3, P.PDE_ADVECTION, P.NUM_FLUX_UPWIND, _adv_state, b_adv=(1.0, 0.5, 0.0),
                             exterior=_adv_state)
    r_ref, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    with Simulation(prob) as sim:
        sim.compute_rhs()
        r = sim.rhs
    assert rel(r, r_ref) <= TOL


def test_taylor_couette_from_a_gmsh_file_on_the_device(gpu_lib, tmp_path):
    """The reference's curved-boundary workflow on the device: a gmsh annulus with curved codes (20113 rotating
    wall inside, 20112 diabatic wall outside) and random local frames -> reader and connectivity -> the blended
    geometry of its curved faces (dgpu_blend_geometry) -> a Navier-Stokes context from the geometry coefficients:
    residual and RK steps against the oracle on the same problem (noise-floor rule of test_gpu_ns.py)."""
    from dpgsolver_gb300.solver import Simulation, blend_geometry
    path = tmp_path / "annulus.msh"
    G.write_annulus_msh(path, 3, 16, outer=20112, rotate_seed=9)

    def state(x):
        U = P.taylor_couette_state(x[:, 0], x[:, 1], 0.5, 1.0, 1.0, 0.02, 0.72, 1.0, 1.0, 1.0, 0.5).T
        return U * (1.0 + 0.1 * np.sin(3.0 * np.arctan2(x[:, 1], x[:, 0])))[:, None]

    def wall(x):
        r, th = np.hypot(x[:, 0], x[:, 1]), np.arctan2(x[:, 1], x[:, 0])
        return np.stack([np.ones_like(r), -np.sin(th) * r, np.cos(th) * r, np.full_like(r, 1.0 / P.GM1 + 0.125)], 1)
    ns = {"viscosity": P.VISCOSITY_CONSTANT, "mu": 0.02, "Pr": 0.72, "r_s": 1.0, "dTdn": 0.5}
    prob = G.gmsh_tp_problem(path, 2, 3, P.PDE_NAVIER_STOKES, P.NUM_FLUX_ROE_PIKE, state, exterior=wall, ns=ns,
                             blend=blend_geometry)
    o = oracle.Oracle(prob)
    r_ref, _ = o.compute_rhs(prob.sol)
    floor = 0.0
    for seed in range(3):
        noisy = prob.sol * (1.0 + np.random.default_rng(seed).choice([-1.0, 1.0], prob.sol.shape) * 2.0 ** -52)
        floor = max(floor, rel(o.compute_rhs(noisy)[0], r_ref))
    s_ref = prob.sol.copy()
    for _ in range(3):
        s_ref, _, _ = o.ssp_rk3_step(s_ref, prob.dt)
    with Simulation(prob, device_geometry=True) as sim:
        sim.compute_rhs()
        r = sim.rhs
        sim.ssp_rk3_steps(prob.dt, 3)
        s = sim.sol_coef
    assert rel(r, r_ref) <= max(TOL, 4.0 * floor)
    assert rel(s, s_ref) <= TOL
