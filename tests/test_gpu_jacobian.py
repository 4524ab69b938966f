"""Block-sparse Jacobian (dgpu_jacobian_bsr) against the oracle's complex-step Jacobian, the reference's own
linearisation (compute_lhs_cmplx_step_dg, test_support_solve_dg.c:83-110), column by column.

Both are exact to rounding, so the bar is the residual's: <= 1e-12 normwise relative over the whole matrix. The
raw form (the reference's lhs, before M^-1) is checked against the oracle's matrix multiplied by each volume's mass
matrix. States are perturbed additively by 1e-2 so that no face node sits on a kink of the numerical fluxes.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12

CASES = {
    "adv2d_p2_4": lambda: P.advection_2d(4, 2),
    "vortex2d_roe_p2_3": lambda: P.euler_vortex_2d(3, 2),
    # n = 2 periodic: both x-neighbours of a volume are the same volume
    "hex_lf_p1_2": lambda: P.euler_hex_3d(2, 1),
    "hex_roe_p2_2": lambda: P.euler_hex_3d(2, 2, num_flux=P.NUM_FLUX_ROE_PIKE),
    "channel2d_roe_p2_3": lambda: P.euler_channel_2d(3, 2),
    "duct3d_roe_p1_2": lambda: P.euler_duct_3d(2, 1),
    "subduct2d_roe_p2_3": lambda: P.euler_subsonic_duct(2, 3, 2),
    "advbox2d_p2_3": lambda: P.advection_box_2d(3, 2),
}


def _base(prob, seed=3):
    rng = np.random.default_rng(seed)
    return prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)


def _dense(row_ptr, col_idx, vals, nb):
    n = (len(row_ptr) - 1) * nb
    A = np.zeros((n, n))
    for v in range(len(row_ptr) - 1):
        for j in range(row_ptr[v], row_ptr[v + 1]):
            w = col_idx[j]
            A[v * nb:(v + 1) * nb, w * nb:(w + 1) * nb] = vals[j]
    return A


def _complex_step_jacobian(prob, base):
    o = oracle.Oracle(prob)
    n = base.size
    J = np.empty((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1e-30
        _, ri = o.compute_rhs_cmplx(base, e.reshape(base.shape))
        J[:, j] = ri.ravel() / 1e-30
    return J, o


def _mass_rows(prob, o, J):
    """kron(I_var, M_v) applied to each volume's block row: the raw residual's Jacobian."""
    nv, nvar, nvs = prob.sol.shape
    nb = nvar * nvs
    out = np.empty_like(J)
    for v in range(nv):
        M = np.kron(np.eye(nvar), np.linalg.inv(o.m_inv(v)))
        out[v * nb:(v + 1) * nb] = M @ J[v * nb:(v + 1) * nb]
    return out


@pytest.mark.parametrize("name", sorted(CASES))
def test_jacobian_matches_complex_step(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    base = _base(prob)
    J_cs, o = _complex_step_jacobian(prob, base)
    with Simulation(prob) as sim:
        nb, nnz, n_col = sim.jacobian_structure()
        rp, ci, vals = sim.jacobian(base, raw=False)
        rp2, ci2, vals_raw = sim.jacobian(base, raw=True)
    assert nb == prob.n_var * prob.ops.n_vs
    # structure: each volume and its distinct face neighbours, ascending
    fv = prob.mesh.face_vol
    for v in range(prob.n_volumes):
        nbrs = {v} | {int(fv[f, 1 - s]) for f in range(len(fv)) for s in range(2)
                      if fv[f, s] == v and fv[f, 1 - s] >= 0}
        assert list(ci[rp[v]:rp[v + 1]]) == sorted(nbrs)
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2)
    A = _dense(rp, ci, vals, nb)
    assert np.max(np.abs(A - J_cs)) <= TOL * np.max(np.abs(J_cs))
    J_raw = _mass_rows(prob, o, J_cs)
    A_raw = _dense(rp, ci, vals_raw, nb)
    assert np.max(np.abs(A_raw - J_raw)) <= TOL * np.max(np.abs(J_raw))


def test_jacobian_times_vector_matches_jvp_and_device_output(gpu_lib):
    """On a mesh too large for a dense check: the block-sparse product with a direction equals dgpu_jvp's, and
    blocks written straight to device memory equal the host copy bit for bit."""
    import torch
    from dpgsolver_gb300.solver import Simulation
    prob = P.euler_hex_3d(3, 3)
    base = _base(prob, 7)
    d = np.random.default_rng(8).standard_normal(prob.sol.shape)
    with Simulation(prob) as sim:
        nb, nnz, n_col = sim.jacobian_structure()
        rp, ci, vals = sim.jacobian(base, raw=False)
        dev = torch.empty((nnz, nb, nb), dtype=torch.float64, device="cuda")
        sim.jacobian(base, raw=False, values_ptr=dev.data_ptr())
        torch.cuda.synchronize()
        _, jv = sim.jvp(base, d)
    assert np.array_equal(dev.cpu().numpy(), vals)
    x = d.reshape(prob.n_volumes, nb)
    y = np.zeros_like(x)
    for v in range(prob.n_volumes):
        for j in range(rp[v], rp[v + 1]):
            y[v] += vals[j] @ x[ci[j]]
    assert np.max(np.abs(y.ravel() - jv.ravel())) <= TOL * np.max(np.abs(jv))
    assert n_col <= 32   # greedy distance-2 colouring of the 6-neighbour periodic lattice
