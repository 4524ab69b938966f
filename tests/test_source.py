"""The source term (compute_source_rhs_dg_like, src/simulation/solvers/compute_rlhs.c:47-57) in the oracle and the
host set-up of the reference's steady advection case (steady/default, solution_advection_default_T.c).

The oracle's residual with the source is pinned to the reference's own output by the golden fixture
tests/golden/reference_c1_source.npz (test_reference_parity.py runs it with the other fixtures). Here: the source
is what closes the gap to that fixture, and on the non-periodic box, where u is the steady solution, the residual of
u falls as h^p (the source balances the advection operator up to the discretisation error) while without the source
it stays O(1).
"""
import os

import numpy as np
import pytest

import oracle
import oracle.reference as R
from dpgsolver_gb300.host import problem as P


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_source_closes_the_gap_to_the_reference():
    ref = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_c1_source.npz")))
    prob = R.with_reference_inputs(R.host_problem("c1_source"), ref)
    assert _rel(oracle.Oracle(prob).compute_rhs(prob.sol)[0], ref["rhs"]) <= 1e-12
    prob.source_vc = None
    assert _rel(oracle.Oracle(prob).compute_rhs(prob.sol)[0], ref["rhs"]) > 1e-3


@pytest.mark.parametrize("p", [1, 2, 3])
def test_steady_residual_converges_at_order_p(p):
    norms = []
    for n in (8, 16):
        prob = P.advection_default_2d(n, p, periodic=False)
        r, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
        norms.append(float(np.sqrt(np.mean(r ** 2))))
    assert norms[0] / norms[1] >= 0.9 * 2 ** p, norms
    prob = P.advection_default_2d(8, p, periodic=False)
    prob.source_vc = None
    r, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    assert float(np.sqrt(np.mean(r ** 2))) > 0.5


def test_source_shape_is_the_state_shape():
    prob = P.advection_default_2d(4, 2)
    assert prob.source_vc.shape == prob.sol.shape
