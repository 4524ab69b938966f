"""The CUDA path, through the C ABI, against outputs of the reference itself.

The golden fixtures tests/golden/reference_*.npz hold what the reference's own compute_rhs and time_step_ssp_rk_33
computed (tests/golden/make_ref_golden.py; the reference is compiled from its sources, it is not a restatement).
The GPU is given exactly what a caller packing the reference's Solver_Volume / Solver_Face lists would pass: the
reference's metric terms, Jacobians, normals and initial state. Its residual and its SSP-RK3 states must match
the reference's to 1e-12 normwise relative error: the advection configuration at its stated size (QUAD 16^2,
p = 2, 100 steps) and the curved Euler vortex (Roe and Lax-Friedrichs, p = 1, 3, 4; 1000 Roe steps on 8^2).
"""
import os

import numpy as np
import pytest

import oracle.reference as R

pytestmark = pytest.mark.gpu
TOL = 1e-12
CASES = [c for c in R.CASES if c != "c2"]


def _fixture(name):
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", f"reference_{name}.npz")))


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name", CASES)
def test_residual_matches_reference(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    ref = _fixture(name)
    prob = R.with_reference_inputs(R.host_problem(name), ref)
    with Simulation(prob) as sim:
        mx = sim.compute_rhs()
        r = sim.rhs
    assert _rel(r, ref["rhs"]) <= TOL
    assert abs(mx - float(ref["max_rhs"])) <= TOL * float(ref["max_rhs"])


@pytest.mark.parametrize("name", CASES)
def test_rk3_steps_match_reference(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    ref = _fixture(name)
    prob = R.with_reference_inputs(R.host_problem(name), ref)
    with Simulation(prob) as sim:
        sim.ssp_rk3_steps(float(ref["dt"]), int(ref["steps"]))
        s = sim.sol_coef
    assert _rel(s, ref["sol_steps"]) <= TOL


@pytest.mark.parametrize("name", ["c1", "c2_n8"])
def test_host_buffer_step_matches_reference(gpu_lib, name):
    """The drop-in for compute_rhs_dg on the caller's host sol_coef (dgpu_compute_rhs_host)."""
    from dpgsolver_gb300.solver import Simulation
    ref = _fixture(name)
    prob = R.with_reference_inputs(R.host_problem(name), ref)
    with Simulation(prob) as sim:
        r, mx = sim.compute_rhs_host(prob.sol)
    assert _rel(r, ref["rhs"]) <= TOL
    assert abs(mx - float(ref["max_rhs"])) <= TOL * float(ref["max_rhs"])
