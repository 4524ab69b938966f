"""Seeded synthetic DG problems (mesh + operators + geometry + state) for the explicit residual path.

These stand in for the reference's own set-up (mesh reading, element operators, geometry, initial
solution). The workloads are the ones the residual path is benchmarked and parity-tested on:

* ``advection_2d``   straight periodic QUAD mesh on [-1,1]^2, p=2, b=(1,0.5), upwind, u0 = sin(pi x) sin(pi y);
* ``euler_vortex_2d`` curved periodic QUAD mesh on [0,10]^2 (x,y += 0.05 sin(pi x/5) sin(pi y/5)), p=3, Roe-Pike,
  isentropic vortex of strength 5 at (5,5) on the free stream (rho,u,v,p)=(1,1,1,1);
* ``euler_hex_3d``   curved periodic HEX mesh on [0,10]^3 with a sinusoidal interior mapping of amplitude 0.03,
  p=3, Lax-Friedrichs (or Roe-Pike), a z-axis isentropic vortex plus seeded uniform density perturbations of 1e-3.

The isentropic vortex is the standard published one (Shu, 1998), not the reference's periodic_vortex case.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .element import TPOperatorSet, gauss_lobatto, lagrange_matrix, kron_tp
from .geometry import TPGeometry, apply_nodes, sinusoidal_deform_2d, sinusoidal_deform_3d
from .mesh import StructuredMesh

PDE_ADVECTION = 1
PDE_EULER = 3
NUM_FLUX_UPWIND = 11
NUM_FLUX_ROE_PIKE = 31
NUM_FLUX_LAX_FRIEDRICHS = 32
GAMMA = 1.4
GM1 = 0.4


@dataclass
class DGProblem:
    name: str
    d: int
    pde: int
    num_flux: int
    positivity: bool
    b_adv: np.ndarray
    ops: TPOperatorSet
    mesh: StructuredMesh
    geom: TPGeometry
    sol: np.ndarray          # (n_volumes, n_var, n_vs): per volume the reference's (n_vs x n_var) 'C' block
    dt: float
    n_steps: int
    meta: dict = field(default_factory=dict)

    @property
    def n_var(self) -> int:
        return self.sol.shape[1]

    @property
    def n_volumes(self) -> int:
        return self.mesh.n_volumes

    @property
    def n_state(self) -> int:
        return int(self.sol.size)

    def nc_fc(self) -> np.ndarray:
        """Right-trace gather permutation per face (identity for these aligned structured meshes)."""
        return np.tile(np.arange(self.ops.n_fc, dtype=np.int32), (self.mesh.n_faces, 1))

    def faces_on_plane(self, axis: int = 2) -> np.ndarray:
        """Faces lying on the plane x_axis = lo[axis] (the periodic seam), with side 0 on the plane's + side."""
        lf = 2 * axis
        sel = (self.mesh.face_lf[:, 0] == lf) & (self.mesh.ijk[self.mesh.face_vol[:, 0], axis] == 0)
        return np.nonzero(sel)[0].astype(np.int32)

    def solution_node_xyz(self) -> np.ndarray:
        """Physical coordinates of the solution (GLL) nodes, (n_volumes, n_vs, d)."""
        xg1, _ = gauss_lobatto(self.geom.p_g + 1)
        L = kron_tp([lagrange_matrix(xg1, self.ops.x_vs)] * self.d)
        return apply_nodes(L, self.geom.X_geom)


def flat_arrays(prob) -> dict:
    """The mesh in the general (multi-group) flat layout the C ABIs take: per-volume blocks concatenated in
    volume-list order, per-face blocks in face-list order. Works for uniform DGProblem and MixedTPProblem."""
    if hasattr(prob, "flat"):
        return prob.flat()
    g = prob.geom
    nf = prob.mesh.n_faces
    return {
        "groups": [prob.ops],
        "vol_group": np.zeros(prob.n_volumes, dtype=np.int32),
        "face_q": np.full(nf, prob.ops.q, dtype=np.int32),
        "metrics_vc": np.ascontiguousarray(np.transpose(g.metrics_vc, (0, 3, 2, 1))).ravel(),
        "jacobian_det_vc": np.ascontiguousarray(g.jacobian_det_vc).ravel(),
        "normals_fc": np.ascontiguousarray(g.normals_fc).ravel(),
        "jacobian_det_fc": np.ascontiguousarray(g.jacobian_det_fc).ravel(),
        "nc_fc": prob.nc_fc().ravel(),
        "sol": np.ascontiguousarray(prob.sol).ravel(),
    }


def stable_dt(prob: "DGProblem", cfl: float = 0.1) -> float:
    """dt = cfl * h / ((2p + 1) * max(|V| + c)) over the solution nodes of the current state."""
    d = prob.d
    U = prob.sol
    rho = U[:, 0]
    vel = U[:, 1:1 + d] / rho[:, None]
    V2 = np.sum(vel * vel, axis=1)
    p = GM1 * (U[:, d + 1] - 0.5 * rho * V2)
    lam = float(np.max(np.sqrt(V2) + np.sqrt(GAMMA * p / rho)))
    h = float(np.min(prob.mesh.h))
    return cfl * h / ((2 * prob.ops.p + 1) * lam)


def primitive_to_conserved(d, rho, vel, p):
    E = p / GM1 + 0.5 * rho * np.sum(vel * vel, axis=0)
    return np.stack([rho] + [rho * vel[k] for k in range(d)] + [E], axis=0)


def isentropic_vortex(xy, x0, y0, beta, u_inf=1.0, v_inf=1.0):
    """Shu's isentropic vortex on free stream (rho, u, v, p) = (1, u_inf, v_inf, 1)."""
    dx = xy[..., 0] - x0
    dy = xy[..., 1] - y0
    r2 = dx * dx + dy * dy
    e = np.exp(0.5 * (1.0 - r2))
    du = -beta / (2.0 * math.pi) * dy * e
    dv = beta / (2.0 * math.pi) * dx * e
    dT = -GM1 * beta * beta / (8.0 * GAMMA * math.pi * math.pi) * np.exp(1.0 - r2)
    T = 1.0 + dT
    rho = T ** (1.0 / GM1)
    p = rho ** GAMMA
    return rho, u_inf + du, v_inf + dv, p


def _pack_state(U):
    """U: (n_var, n_volumes, n_vs) -> (n_volumes, n_var, n_vs) contiguous."""
    return np.ascontiguousarray(np.transpose(U, (1, 0, 2)))


def advection_2d(n: int = 16, p: int = 2, b=(1.0, 0.5), cfl: float = 0.1, n_steps: int = 100) -> DGProblem:
    mesh = StructuredMesh(2, n, -1.0, 1.0)
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, deform=None)
    b_adv = np.array([b[0], b[1], 0.0])
    prob = DGProblem("advection_2d", 2, PDE_ADVECTION, NUM_FLUX_UPWIND, False, b_adv, ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 1, ops.n_vs)), dt=0.0, n_steps=n_steps)
    xyz = prob.solution_node_xyz()
    prob.sol[:, 0, :] = np.sin(math.pi * xyz[..., 0]) * np.sin(math.pi * xyz[..., 1])
    h = float(mesh.h[0])
    prob.dt = cfl * h / float(np.linalg.norm(b_adv))
    prob.meta.update(n=n, p=p, h=h, cfl=cfl)
    return prob


def euler_vortex_2d(n: int = 64, p: int = 3, num_flux: int = NUM_FLUX_ROE_PIKE, amplitude: float = 0.05,
                    dt: float | None = None, n_steps: int = 1000) -> DGProblem:
    L = 10.0
    mesh = StructuredMesh(2, n, 0.0, L)
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, deform=sinusoidal_deform_2d(amplitude, L), curved=True)
    prob = DGProblem("euler_vortex_2d", 2, PDE_EULER, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 4, ops.n_vs)), dt=0.0, n_steps=n_steps)
    xyz = prob.solution_node_xyz()
    rho, u, v, pr = isentropic_vortex(xyz, 5.0, 5.0, 5.0)
    U = primitive_to_conserved(2, rho, np.stack([u, v]), pr)
    prob.sol = _pack_state(U)
    prob.dt = stable_dt(prob) if dt is None else dt
    prob.meta.update(n=n, p=p, amplitude=amplitude)
    return prob


def euler_hex_3d(n: int = 32, p: int = 3, num_flux: int = NUM_FLUX_LAX_FRIEDRICHS, amplitude: float = 0.03,
                 seed: int = 0, perturb: float = 1e-3, dt: float | None = None, n_steps: int = 200) -> DGProblem:
    L = 10.0
    mesh = StructuredMesh(3, n, 0.0, L)
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, deform=sinusoidal_deform_3d(amplitude, L), curved=True)
    prob = DGProblem("euler_hex_3d", 3, PDE_EULER, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 5, ops.n_vs)), dt=0.0, n_steps=n_steps)
    xyz = prob.solution_node_xyz()
    rho, u, v, pr = isentropic_vortex(xyz, 5.0, 5.0, 5.0)
    rng = np.random.default_rng(seed)
    rho = rho + perturb * rng.uniform(-1.0, 1.0, size=rho.shape)
    w = np.zeros_like(u)
    U = primitive_to_conserved(3, rho, np.stack([u, v, w]), pr)
    prob.sol = _pack_state(U)
    prob.dt = stable_dt(prob) if dt is None else dt
    prob.meta.update(n=n, p=p, amplitude=amplitude, seed=seed)
    return prob


def constant_state(prob: DGProblem, values) -> np.ndarray:
    """Free-stream state (same conserved values at every node), in the problem's layout."""
    s = np.empty_like(prob.sol)
    for k, val in enumerate(values):
        s[:, k, :] = val
    return s
