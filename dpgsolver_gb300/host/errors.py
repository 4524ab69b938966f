"""Error functionals of a solved state (harness side, as the reference computes them after a run).

``l2_entropy_error`` follows constructor_Error_CE_euler_entropy (test_case/compute_error/compute_error_euler.c:
135-180) and the L2 reduction of compute_error.c: the entropy variable s = log(p rho^-gamma) (compute_entropy,
solution/euler/solution_euler.c:72-91) is evaluated at the volume cubature nodes, the squared difference to the
exact entropy is integrated with w_vc J_vc over every volume, and the result is sqrt(sum / domain volume).
"""
from __future__ import annotations

import numpy as np

from .problem import GAMMA, GM1


def entropy_at_cubature(prob, sol):
    """s = log(p rho^-gamma) at the volume cubature nodes, (n_volumes, n_vc), for a uniform TP Euler problem."""
    V = prob.ops.cv0_vs_vc()                               # (n_vc, n_vs)
    W = np.einsum("cn,vkn->vkc", V, np.asarray(sol))       # conserved variables at the nodes
    d = prob.d
    rho = W[:, 0]
    m2 = np.sum(W[:, 1:1 + d] ** 2, axis=1)
    p = GM1 * (W[:, d + 1] - 0.5 * m2 / rho)
    return np.log(p * rho ** (-GAMMA))


def l2_entropy_error(prob, sol, s_exact: float = 0.0) -> float:
    """sqrt(sum_v int_v (s - s_exact)^2 / |Omega|). The isentropic vortex on a (rho, p) = (1, 1) free stream has
    p = rho^gamma everywhere, so its exact entropy is s = 0 at all times."""
    s = entropy_at_cubature(prob, sol)
    wJ = prob.ops.w_vc[None, :] * prob.geom.jacobian_det_vc
    return float(np.sqrt(np.sum(wJ * (s - s_exact) ** 2) / np.sum(wJ)))


def kinetic_energy(prob, sol) -> float:
    """Volume-averaged kinetic energy (1/|Omega|) int rho |u|^2 / 2 (the Taylor-Green vortex's dissipation
    diagnostic), by the volume cubature of a uniform TP problem."""
    V = prob.ops.cv0_vs_vc()
    W = np.einsum("cn,vkn->vkc", V, np.asarray(sol))
    d = prob.d
    ek = 0.5 * np.sum(W[:, 1:1 + d] ** 2, axis=1) / W[:, 0]
    wJ = prob.ops.w_vc[None, :] * prob.geom.jacobian_det_vc
    return float(np.sum(wJ * ek) / np.sum(wJ))
