"""Boundary faces on the CUDA path (dgpu_create with bc_fc / bc_state_fc) against the CPU oracle.

The residual, SSP-RK3 steps, the forward linearisation (against the oracle's complex step) and the adjoint (the
transpose of the forward one) on bounded meshes: slip walls, Riemann, supersonic inflow/outflow, back pressure,
total temperature/pressure and upwind advection boundaries (the reference's boundary values, test_case/boundary/boundary_euler_T.c and
boundary_advection_T.c). Tolerances as in test_gpu_parity.py: <= 1e-12 normwise relative.
"""
import ctypes

import numpy as np
import pytest

import oracle
from dpgsolver_gb300 import _lib
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12

CASES = {
    "channel2d_roe_p3_8": lambda: P.euler_channel_2d(8, 3),
    "channel2d_lf_p2_6": lambda: P.euler_channel_2d(6, 2, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "riemann2d_lf_p3_8": lambda: P.euler_riemann_2d(8, 3),
    "riemann2d_roe_p4_5": lambda: P.euler_riemann_2d(5, 4, num_flux=P.NUM_FLUX_ROE_PIKE),
    "duct3d_roe_p2_4": lambda: P.euler_duct_3d(4, 2),
    "duct3d_lf_p3_4": lambda: P.euler_duct_3d(4, 3, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "duct3d_roe_p1_6": lambda: P.euler_duct_3d(6, 1),
    "advbox2d_p2_8": lambda: P.advection_box_2d(8, 2),
    "advbox2d_p4_4": lambda: P.advection_box_2d(4, 4, b=(-0.6, 1.1)),
    "subduct2d_roe_p3_8": lambda: P.euler_subsonic_duct(2, 8, 3),
    "subduct3d_lf_p2_4": lambda: P.euler_subsonic_duct(3, 4, 2, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "subduct3d_roe_p3_4": lambda: P.euler_subsonic_duct(3, 4, 3),
    # many CTAs: boundary and interior faces interleaved across the whole grid
    "duct3d_roe_p3_12": lambda: P.euler_duct_3d(12, 3),
}


def rel_err(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", sorted(CASES))
def test_bc_residual_matches_oracle(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    r_ref, mx_ref = oracle.Oracle(prob).compute_rhs(prob.sol)
    with Simulation(prob) as sim:
        mx = sim.compute_rhs()
        r = sim.rhs
    assert rel_err(r, r_ref) <= TOL
    assert abs(mx - mx_ref) <= TOL * mx_ref


@pytest.mark.parametrize("name", ["channel2d_roe_p3_8", "riemann2d_lf_p3_8", "duct3d_roe_p2_4", "advbox2d_p2_8",
                                  "subduct3d_roe_p3_4"])
def test_bc_rk3_steps_match_oracle(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    ref = oracle.Oracle(prob)
    s_ref = prob.sol.copy()
    for _ in range(5):
        s_ref, mx_ref, _ = ref.ssp_rk3_step(s_ref, prob.dt)
    with Simulation(prob) as sim:
        mx = sim.ssp_rk3_steps(prob.dt, 5)
        s = sim.sol_coef
    assert rel_err(s, s_ref) <= TOL
    assert abs(mx - mx_ref) <= 1e-10 * mx_ref


def test_bc_free_stream_preserved_on_gpu(gpu_lib):
    """Streams that satisfy every boundary condition are steady: Riemann sides with the free stream as exterior,
    slip walls with a tangential stream, the supersonic duct with its Mach 2 stream, the subsonic duct (total
    temperature/pressure inflow, back-pressure outflow) with the stream its BC data come from."""
    from dpgsolver_gb300.solver import Simulation

    def stream(prob, rho, vel, p):
        vel = np.asarray(vel, dtype=np.float64)
        return P.constant_state(prob, [rho] + list(rho * vel) + [p / P.GM1 + 0.5 * rho * float(vel @ vel)])
    u0, u1 = 2.0 * np.sqrt(P.GAMMA), 0.4 * np.sqrt(P.GAMMA)
    for prob, st in ((P.euler_riemann_2d(8, 3), (1.0, (1.0, 1.0), 1.0)),
                     (P.euler_channel_2d(8, 3), (1.0, (0.8, 0.0), 1.0)),
                     (P.euler_duct_3d(4, 3), (1.0, (u0, 0.0, 0.0), 1.0)),
                     (P.euler_subsonic_duct(3, 4, 3), (1.0, (u1, 0.0, 0.0), 1.0))):
        with Simulation(prob) as sim:
            sim.upload_state(stream(prob, *st))
            assert sim.compute_rhs() < 1e-10


def _perturbed(prob, seed):
    rng = np.random.default_rng(seed)
    return prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape), rng.standard_normal(prob.sol.shape)


@pytest.mark.parametrize("name", ["channel2d_roe_p3_8", "riemann2d_roe_p4_5", "duct3d_lf_p3_4", "duct3d_roe_p2_4",
                                  "advbox2d_p2_8", "subduct2d_roe_p3_8", "subduct3d_lf_p2_4"])
def test_bc_jvp_matches_complex_step(gpu_lib, name):
    """The dual-number boundary values against the oracle's complex-step ones (the reference's linearisation)."""
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    base, dirn = _perturbed(prob, 5)
    r_ref, ri = oracle.Oracle(prob).compute_rhs_cmplx(base, 1e-30 * dirn)
    with Simulation(prob) as sim:
        r, jv = sim.jvp(base, dirn)
    assert rel_err(r, r_ref) <= TOL
    assert rel_err(jv, ri / 1e-30) <= TOL


@pytest.mark.parametrize("name", ["channel2d_roe_p3_8", "riemann2d_lf_p3_8", "duct3d_roe_p2_4", "advbox2d_p2_8",
                                  "subduct2d_roe_p3_8"])
def test_bc_vjp_is_the_transpose_of_the_jvp(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    base, dirn = _perturbed(prob, 9)
    v = np.random.default_rng(10).standard_normal(prob.sol.shape)
    with Simulation(prob) as sim:
        _, jv = sim.jvp(base, dirn)
        sim.vjp_forward(base)
        g = sim.vjp_backward(v)
    lhs, rhs = float(np.sum(v * jv)), float(np.sum(g * dirn))
    assert abs(lhs - rhs) <= 1e-12 * np.sqrt(np.sum(v * v) * np.sum(jv * jv))


def test_bc_create_errors(gpu_lib):
    """Boundary faces without BC arrays, and BC codes the library does not provide, are refused at creation."""
    from dpgsolver_gb300.solver import Simulation
    prob = P.euler_channel_2d(4, 2)
    bc, bcs = prob.bc, prob.bc_state
    prob.bc, prob.bc_state = None, None
    with pytest.raises(_lib.DGPUError) as e:
        Simulation(prob)
    assert e.value.status == 1
    for code in (111, 113, 41, 999):      # no-slip walls (Navier-Stokes); an advection code on Euler; junk
        prob.bc, prob.bc_state = np.where(bc > 0, code, 0).astype(np.int32), bcs
        with pytest.raises(_lib.DGPUError) as e:
            Simulation(prob)
        assert e.value.status == 2
    prob.bc = np.where(bc > 0, 103, 0).astype(np.int32)            # back pressure without its BC data
    with pytest.raises(_lib.DGPUError) as e:
        Simulation(prob)
    assert e.value.status == 1
    prob.bc = np.where(bc > 0, 20000 + 102, 0).astype(np.int32)   # curved slip wall: the same boundary value
    with Simulation(prob) as sim:
        mx = sim.compute_rhs()
    prob.bc = bc
    _, mx_ref = oracle.Oracle(prob).compute_rhs(prob.sol)
    assert abs(mx - mx_ref) <= TOL * mx_ref


def test_bc_in_batched_context_and_refused_by_noalloc(gpu_lib):
    """The batched context takes boundary faces (a uniform mesh as one group matches the oracle); the
    no-allocation entry refuses them."""
    from dpgsolver_gb300.solver import BatchSimulation
    prob = P.euler_channel_2d(4, 2)
    r_ref, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    with BatchSimulation(prob) as sim:
        sim.compute_rhs()
        r = sim.rhs
    assert np.max(np.abs(np.reshape(r, r_ref.shape) - r_ref)) <= TOL * np.max(np.abs(r_ref))
    phys = _lib.Physics()
    phys.d, phys.pde, phys.num_flux = 2, prob.pde, prob.num_flux
    tp = _lib.TPOperators()
    tp.elem_type, tp.p = prob.ops.e_type, prob.ops.p
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (prob.ops.cv0_1d, prob.ops.cv1_1d,
                                                                 prob.ops.cv0_bnd_1d, prob.ops.w_vc_1d)]
    tp.cv0_vs_vc, tp.cv1_vs_vc, tp.cv0_vs_fc, tp.w_vc = [a.ctypes.data_as(_lib.c_double_p) for a in keep]
    m = _lib.Mesh()
    m.n_volumes, m.n_faces = prob.n_volumes, prob.mesh.n_faces
    bc = np.ascontiguousarray(prob.bc, dtype=np.int32)
    m.bc_fc = bc.ctypes.data_as(_lib.c_int_p)
    dummy = ctypes.c_void_p(1)
    st = gpu_lib.dgpu_compute_rhs_noalloc(ctypes.byref(phys), ctypes.byref(tp), ctypes.byref(m), dummy, dummy,
                                          None, None)
    assert st == 2
    assert b"boundary" in gpu_lib.dgpu_last_error(None)
