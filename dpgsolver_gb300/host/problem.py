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
PDE_NAVIER_STOKES = 4
VISCOSITY_CONSTANT = 101
VISCOSITY_SUTHERLAND = 102
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
    bc: np.ndarray | None = None          # (n_faces,) BC code of each face (definitions_bc.h), 0 on interior faces
    bc_state: np.ndarray | None = None    # (n_faces, n_fc, n_var) exterior conserved state at the face nodes
    bc_data: tuple | None = None          # (p_back, t_total, p_total, r_s): BC_Data of boundary_euler_T.c:44-49
    ns: dict | None = None                # Navier-Stokes: {"viscosity": 101|102, "mu", "Pr", "r_s"}
    source_vc: np.ndarray | None = None   # (n_volumes, n_var, n_vc): the test case's source at the volume cubature
                                          # nodes (compute_source_rhs_dg_like), before the J scaling

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
        """Right-trace gather permutation per face: the mesh's own (a mesh read from a file, whose neighbouring
        volumes may see a face in different orientations), else the identity (aligned structured meshes)."""
        if hasattr(self.mesh, "nc_fc"):
            return self.mesh.nc_fc(self.ops.q)
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
        "bc_fc": None if prob.bc is None else np.ascontiguousarray(prob.bc, dtype=np.int32),
        "bc_state_fc": None if prob.bc_state is None else np.ascontiguousarray(prob.bc_state).ravel(),
        "bc_data": prob.bc_data,
        "source_vc": None if prob.source_vc is None else np.ascontiguousarray(prob.source_vc).ravel(),
    }


def stable_dt(prob: "DGProblem", cfl: float = 0.1, h: float | None = None) -> float:
    """dt = cfl * h / ((2p + 1) * max(|V| + c)) over the solution nodes of the current state; with viscosity also
    at most cfl * h^2 / ((2p + 1)^2 * max(gamma mu / (Pr rho))) (the heat-flux diffusivity bounds the momentum one
    for Pr < gamma). h: the smallest physical volume size (the structured mesh's own spacing by default)."""
    d = prob.d
    U = prob.sol
    rho = U[:, 0]
    vel = U[:, 1:1 + d] / rho[:, None]
    V2 = np.sum(vel * vel, axis=1)
    p = GM1 * (U[:, d + 1] - 0.5 * rho * V2)
    lam = float(np.max(np.sqrt(V2) + np.sqrt(GAMMA * p / rho)))
    h = float(np.min(prob.mesh.h)) if h is None else float(h)
    k = 2 * prob.ops.p + 1
    dt = cfl * h / (k * lam)
    if prob.ns is not None and prob.ns["mu"] > 0.0:
        mu = prob.ns["mu"]
        if prob.ns["viscosity"] == VISCOSITY_SUTHERLAND:   # 0.08 mu sqrt(T) / (1 + 112 / T) <= 0.08 mu sqrt(T)
            mu *= 0.08 * float(np.sqrt(np.max(p / (rho * prob.ns["r_s"]))))
        nu = GAMMA * mu / (prob.ns["Pr"] * float(np.min(rho)))
        dt = min(dt, cfl * h * h / (k * k * nu))
    return dt


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


# constants of the reference's steady linear-advection case u = sin(M x + A) sin(M y + A)
# (solution_advection_default_T.c:38-39)
SOURCE_M = 2.15
SOURCE_A = 0.23


def advection_default_2d(n: int = 8, p: int = 3, b=(1.0, 0.5), amplitude: float = 0.05, cfl: float = 0.1,
                         n_steps: int = 20, periodic: bool = True) -> DGProblem:
    """The reference's steady linear-advection case with a source ("steady/default",
    solution_advection_default_T.c): u = sin(M x + A) sin(M y + A), source s = b . grad u at the volume cubature
    nodes, on a QUAD mesh of [-1,1]^2 mapped by x, y += amplitude sin(pi x) sin(pi y) (parametric: the mapped faces
    blended into the volumes). The state starts at u on the solution nodes. periodic=False puts upwind boundaries
    (BC_UPWIND) on the four sides with u as the exterior state, where u is the steady solution (the periodic mesh
    leaves a jump of u at the seams, u not being periodic on [-1,1])."""
    mesh = StructuredMesh(2, n, -1.0, 1.0, periodic=(True, True) if periodic else (False, False))
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, deform=sinusoidal_deform_2d(amplitude, 2.0), curved=True, parametric=True)
    b_adv = np.array([b[0], b[1], 0.0])
    prob = DGProblem("advection_default_2d", 2, PDE_ADVECTION, NUM_FLUX_UPWIND, False, b_adv, ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 1, ops.n_vs)), dt=0.0, n_steps=n_steps)
    xyz = prob.solution_node_xyz()
    prob.sol[:, 0, :] = np.sin(SOURCE_M * xyz[..., 0] + SOURCE_A) * np.sin(SOURCE_M * xyz[..., 1] + SOURCE_A)
    x, y = geom.xyz_vc[..., 0], geom.xyz_vc[..., 1]
    sx, cx = np.sin(SOURCE_M * x + SOURCE_A), np.cos(SOURCE_M * x + SOURCE_A)
    sy, cy = np.sin(SOURCE_M * y + SOURCE_A), np.cos(SOURCE_M * y + SOURCE_A)
    prob.source_vc = (b[0] * SOURCE_M * cx * sy + b[1] * SOURCE_M * sx * cy)[:, None, :]
    h = float(mesh.h[0])
    prob.dt = cfl * h / float(np.linalg.norm(b_adv))
    prob.meta.update(n=n, p=p, h=h, cfl=cfl, amplitude=amplitude)
    if periodic:
        return prob

    def ext(xy):
        return (np.sin(SOURCE_M * xy[:, 0] + SOURCE_A) * np.sin(SOURCE_M * xy[:, 1] + SOURCE_A))[:, None]
    return _set_boundaries(prob, {(dd, sd): BC_UPWIND for dd in range(2) for sd in range(2)}, ext)


def euler_vortex_2d(n: int = 64, p: int = 3, num_flux: int = NUM_FLUX_ROE_PIKE, amplitude: float = 0.05,
                    dt: float | None = None, n_steps: int = 1000, parametric: bool = True) -> DGProblem:
    """The curved 2D vortex. parametric: the domain map applied the way the reference applies it to a parametric
    domain (mapped faces blended into the volumes, geometry_T.c:857-874), else to every geometry node."""
    L = 10.0
    mesh = StructuredMesh(2, n, 0.0, L)
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, deform=sinusoidal_deform_2d(amplitude, L), curved=True, parametric=parametric)
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
                 seed: int = 0, perturb: float = 1e-3, dt: float | None = None, n_steps: int = 200,
                 stack: int = 1) -> DGProblem:
    """The curved 3D vortex on [0,10]^3 (n^3 volumes); stack > 1 repeats the box along z (n x n x stack n volumes on
    [0,10]^2 x [0,10 stack], the same map and vortex), the weak-scaling mesh of stack element partitions."""
    L = 10.0
    mesh = StructuredMesh(3, [n, n, n * stack], 0.0, [L, L, L * stack]) if stack > 1 else StructuredMesh(3, n, 0.0, L)
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


# ---- bounded domains: the reference's BC codes (test_case/boundary/definitions_bc.h) ----------------------------
BC_UPWIND = 41
BC_RIEMANN = 101
BC_SLIPWALL = 102
BC_BACKPRESSURE = 103
BC_TOTAL_TP = 104
BC_SUPERSONIC_IN = 105
BC_SUPERSONIC_OUT = 106
BC_NOSLIP_ADIABATIC = 111
BC_NOSLIP_DIABATIC = 112
BC_NOSLIP_ALL_ROTATING = 113


def _set_boundaries(prob: DGProblem, side_bc: dict, exterior) -> DGProblem:
    """bc per face from {(dim, side): code} and the exterior state exterior(xyz (m, d)) -> (m, n_var) at every face
    node (the test case's constructor_sol_bv)."""
    mesh = prob.mesh
    bc = np.zeros(mesh.n_faces, dtype=np.int32)
    bnd = np.nonzero(mesh.face_vol[:, 1] < 0)[0]
    for f in bnd:
        lf = int(mesh.face_lf[f, 0])
        bc[f] = side_bc[(lf // 2, lf % 2)]
    xyz = prob.geom.xyz_fc                                   # (n_faces, n_fc, d)
    ext = exterior(xyz.reshape(-1, prob.d)).reshape(mesh.n_faces, -1, prob.n_var)
    ext[mesh.face_vol[:, 1] >= 0] = 0.0
    prob.bc, prob.bc_state = bc, np.ascontiguousarray(ext)
    return prob


def _uniform_flow(d, rho, vel, p):
    def f(x):
        vv = np.broadcast_to(np.asarray(vel, dtype=np.float64)[:, None], (d, len(x)))
        U = primitive_to_conserved(d, np.full(len(x), rho), vv, np.full(len(x), p))
        return U.T
    return f


def euler_channel_2d(n: int = 8, p: int = 3, num_flux: int = NUM_FLUX_ROE_PIKE, amplitude: float = 0.05) -> DGProblem:
    """The curved isentropic-vortex mesh and state of euler_vortex_2d, periodic in x and bounded in y by slip walls
    (BC_SLIPWALL); the walls stay straight under the sinusoidal mapping."""
    L = 10.0
    mesh = StructuredMesh(2, n, 0.0, L, periodic=(True, False))
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, deform=sinusoidal_deform_2d(amplitude, L), curved=True)
    prob = DGProblem("euler_channel_2d", 2, PDE_EULER, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 4, ops.n_vs)), dt=0.0, n_steps=100)
    xyz = prob.solution_node_xyz()
    rho, u, v, pr = isentropic_vortex(xyz, 5.0, 5.0, 5.0)
    prob.sol = _pack_state(primitive_to_conserved(2, rho, np.stack([u, v]), pr))
    prob.dt = stable_dt(prob)
    return _set_boundaries(prob, {(1, 0): BC_SLIPWALL, (1, 1): BC_SLIPWALL}, _uniform_flow(2, 1.0, (1.0, 1.0), 1.0))


def euler_riemann_2d(n: int = 8, p: int = 3, num_flux: int = NUM_FLUX_LAX_FRIEDRICHS,
                     amplitude: float = 0.05) -> DGProblem:
    """The vortex mesh and state with characteristic (BC_RIEMANN) boundaries on all four sides, the exterior being
    the free stream (rho, u, v, p) = (1, 1, 1, 1)."""
    L = 10.0
    mesh = StructuredMesh(2, n, 0.0, L, periodic=(False, False))
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, deform=sinusoidal_deform_2d(amplitude, L), curved=True)
    prob = DGProblem("euler_riemann_2d", 2, PDE_EULER, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 4, ops.n_vs)), dt=0.0, n_steps=100)
    xyz = prob.solution_node_xyz()
    rho, u, v, pr = isentropic_vortex(xyz, 5.0, 5.0, 5.0)
    prob.sol = _pack_state(primitive_to_conserved(2, rho, np.stack([u, v]), pr))
    prob.dt = stable_dt(prob)
    sides = {(dd, s): BC_RIEMANN for dd in range(2) for s in range(2)}
    return _set_boundaries(prob, sides, _uniform_flow(2, 1.0, (1.0, 1.0), 1.0))


def euler_duct_3d(n: int = 4, p: int = 2, num_flux: int = NUM_FLUX_ROE_PIKE, amplitude: float = 0.03,
                  mach: float = 2.0, seed: int = 0, perturb: float = 0.02) -> DGProblem:
    """Curved HEX box [0,10]^3 with a Mach `mach` stream along x: supersonic inflow at x = 0 (BC_SUPERSONIC_IN),
    supersonic outflow at x = 10 (BC_SUPERSONIC_OUT), slip walls in y (BC_SLIPWALL), characteristic boundaries in z
    (BC_RIEMANN); the state is the stream with seeded smooth perturbations."""
    L = 10.0
    mesh = StructuredMesh(3, n, 0.0, L, periodic=(False, False, False))
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, deform=sinusoidal_deform_3d(amplitude, L), curved=True)
    prob = DGProblem("euler_duct_3d", 3, PDE_EULER, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 5, ops.n_vs)), dt=0.0, n_steps=100)
    xyz = prob.solution_node_xyz()
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0.0, 2.0 * math.pi, size=(5, 3))

    def wave(k):
        s = np.ones(xyz.shape[:2])
        for j in range(3):
            s = s * np.sin(2.0 * math.pi * xyz[..., j] / L + ph[k, j])
        return s
    u0 = mach * math.sqrt(GAMMA)
    vel = np.stack([u0 * (1.0 + perturb * wave(2)), u0 * perturb * wave(3), u0 * perturb * wave(4)])
    prob.sol = _pack_state(primitive_to_conserved(3, 1.0 + perturb * wave(0), vel, 1.0 + perturb * wave(1)))
    prob.dt = stable_dt(prob)
    sides = {(0, 0): BC_SUPERSONIC_IN, (0, 1): BC_SUPERSONIC_OUT, (1, 0): BC_SLIPWALL, (1, 1): BC_SLIPWALL,
             (2, 0): BC_RIEMANN, (2, 1): BC_RIEMANN}
    return _set_boundaries(prob, sides, _uniform_flow(3, 1.0, (u0, 0.0, 0.0), 1.0))


def advection_box_2d(n: int = 8, p: int = 2, b=(1.0, 0.5)) -> DGProblem:
    """advection_2d's state on [-1,1]^2 without periodicity: upwind boundaries (BC_UPWIND) whose exterior state is
    the initial solution sin(pi x) sin(pi y) at the face nodes (inflow sides take it, outflow sides the interior)."""
    mesh = StructuredMesh(2, n, -1.0, 1.0, periodic=(False, False))
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops)
    prob = DGProblem("advection_box_2d", 2, PDE_ADVECTION, NUM_FLUX_UPWIND, False, np.array([b[0], b[1], 0.0]), ops,
                     mesh, geom, sol=np.zeros((mesh.n_volumes, 1, ops.n_vs)), dt=0.0, n_steps=100)
    xyz = prob.solution_node_xyz()
    prob.sol = (np.sin(np.pi * xyz[..., 0]) * np.sin(np.pi * xyz[..., 1]))[:, None, :]
    prob.dt = 0.1 * float(np.min(mesh.h)) / ((2 * p + 1) * float(np.hypot(*b)))

    def ext(x):
        return (np.sin(np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1]))[:, None]
    sides = {(dd, s): BC_UPWIND for dd in range(2) for s in range(2)}
    return _set_boundaries(prob, sides, ext)


def subsonic_duct_state(xyz, d: int, mach: float, perturb: float, seed: int, L: float = 10.0):
    """The subsonic duct's state at points xyz (..., d): the stream (rho, u, p) = (1, mach sqrt(gamma), 1) along x
    with seeded smooth perturbations of relative size perturb. Conserved (d + 2, ...)."""
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0.0, 2.0 * math.pi, size=(d + 2, d))

    def wave(k):
        s = np.ones(xyz.shape[:-1])
        for j in range(d):
            s = s * np.sin(2.0 * math.pi * xyz[..., j] / L + ph[k, j])
        return s
    u0 = mach * math.sqrt(GAMMA)
    vel = np.stack([u0 * (1.0 + perturb * wave(2))] + [u0 * perturb * wave(3 + j) for j in range(d - 1)])
    return primitive_to_conserved(d, 1.0 + perturb * wave(0), vel, 1.0 + perturb * wave(1))


def euler_subsonic_duct(d: int = 2, n: int = 6, p: int = 3, num_flux: int = NUM_FLUX_ROE_PIKE, mach: float = 0.4,
                        amplitude: float = 0.03, seed: int = 0, perturb: float = 0.02) -> DGProblem:
    """Curved QUAD/HEX box [0,10]^d with a subsonic stream along x: total temperature and pressure inflow at x = 0
    (BC_TOTAL_TP), back pressure outflow at x = 10 (BC_BACKPRESSURE), slip walls on the other sides. The BC data
    (p_back, t_total, p_total, r_s) are those of the unperturbed stream (rho, p) = (1, 1), r_s = 1 (T = p / rho), so
    that stream is a steady state; the state is the stream with seeded smooth perturbations."""
    L = 10.0
    mesh = StructuredMesh(d, n, 0.0, L, periodic=(False,) * d)
    ops = TPOperatorSet(mesh.e_type, p)
    deform = sinusoidal_deform_2d(amplitude, L) if d == 2 else sinusoidal_deform_3d(amplitude, L)
    geom = TPGeometry(mesh, ops, deform=deform, curved=True)
    prob = DGProblem(f"euler_subsonic_duct_{d}d", d, PDE_EULER, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, d + 2, ops.n_vs)), dt=0.0, n_steps=100)
    prob.sol = _pack_state(subsonic_duct_state(prob.solution_node_xyz(), d, mach, perturb, seed, L))
    u0 = mach * math.sqrt(GAMMA)
    prob.dt = stable_dt(prob)
    T_tot = 1.0 + 0.5 * GM1 * mach * mach
    prob.bc_data = (1.0, T_tot, T_tot ** (GAMMA / GM1), 1.0)
    sides = {(0, 0): BC_TOTAL_TP, (0, 1): BC_BACKPRESSURE}
    sides.update({(k, s): BC_SLIPWALL for k in range(1, d) for s in range(2)})
    return _set_boundaries(prob, sides, _uniform_flow(d, 1.0, (u0,) + (0.0,) * (d - 1), 1.0))


def euler_supersonic_duct_2d(n: int = 4, p: int = 3, num_flux: int = NUM_FLUX_ROE_PIKE, mach: float = 1.5,
                             seed: int = 0, perturb: float = 0.02) -> DGProblem:
    """Straight QUAD box [0,10]^2 with a supersonic stream along x: supersonic inflow at x = 0 (BC_SUPERSONIC_IN,
    the unperturbed stream (rho, p) = (1, 1) outside), supersonic outflow at x = 10 (BC_SUPERSONIC_OUT), slip walls
    at y = 0 and 10; the state is the stream with seeded smooth perturbations (subsonic_duct_state at this Mach)."""
    L = 10.0
    mesh = StructuredMesh(2, n, 0.0, L, periodic=(False, False))
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops)
    prob = DGProblem("euler_supersonic_duct_2d", 2, PDE_EULER, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 4, ops.n_vs)), dt=0.0, n_steps=100)
    prob.sol = _pack_state(subsonic_duct_state(prob.solution_node_xyz(), 2, mach, perturb, seed, L))
    prob.dt = stable_dt(prob)
    sides = {(0, 0): BC_SUPERSONIC_IN, (0, 1): BC_SUPERSONIC_OUT, (1, 0): BC_SLIPWALL, (1, 1): BC_SLIPWALL}
    return _set_boundaries(prob, sides, _uniform_flow(2, 1.0, (mach * math.sqrt(GAMMA), 0.0), 1.0))


# ---- Navier-Stokes (pde 4: Euler inviscid flux + viscous flux, BR2 second-order numerical flux) ----------------------
def _ns_params(mu, Pr=0.72, viscosity=VISCOSITY_CONSTANT, r_s=1.0):
    return {"viscosity": int(viscosity), "mu": float(mu), "Pr": float(Pr), "r_s": float(r_s)}


def ns_taylor_green(n: int = 8, p: int = 3, Re: float = 1600.0, mach: float = 0.1,
                    num_flux: int = NUM_FLUX_ROE_PIKE, amplitude: float = 0.0, viscosity=VISCOSITY_CONSTANT,
                    dt: float | None = None, n_steps: int = 200) -> DGProblem:
    """The Taylor-Green vortex, the standard viscous DG benchmark: periodic HEX box [0, 2 pi]^3, rho = 1,
    u = sin x cos y cos z, v = -cos x sin y cos z, w = 0, p = 1 / (gamma Ma^2) + (cos 2x + cos 2y)(cos 2z + 2) / 16,
    mu = 1 / Re (unit length and velocity), Pr = 0.72 (Brachet et al., 1983; the published case, not a reference
    input file). amplitude > 0 curves the mesh with the sinusoidal interior mapping."""
    L = 2.0 * math.pi
    mesh = StructuredMesh(3, n, 0.0, L)
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, deform=sinusoidal_deform_3d(amplitude, L) if amplitude > 0 else None,
                      curved=amplitude > 0)
    prob = DGProblem("ns_taylor_green", 3, PDE_NAVIER_STOKES, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 5, ops.n_vs)), dt=0.0, n_steps=n_steps,
                     ns=_ns_params(1.0 / Re, viscosity=viscosity))
    x = prob.solution_node_xyz()
    X, Y, Z = x[..., 0], x[..., 1], x[..., 2]
    rho = np.ones_like(X)
    vel = np.stack([np.sin(X) * np.cos(Y) * np.cos(Z), -np.cos(X) * np.sin(Y) * np.cos(Z), np.zeros_like(X)])
    pr = 1.0 / (GAMMA * mach * mach) + (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0) / 16.0
    prob.sol = _pack_state(primitive_to_conserved(3, rho, vel, pr))
    prob.dt = stable_dt(prob) if dt is None else dt
    prob.meta.update(n=n, p=p, Re=Re, mach=mach)
    return prob


def ns_vortex_2d(n: int = 8, p: int = 3, mu: float = 0.01, num_flux: int = NUM_FLUX_ROE_PIKE,
                 amplitude: float = 0.05, viscosity=VISCOSITY_CONSTANT) -> DGProblem:
    """The curved periodic 2D vortex of euler_vortex_2d with viscosity mu (Pr = 0.72)."""
    prob = euler_vortex_2d(n, p, num_flux=num_flux, amplitude=amplitude)
    prob.name = "ns_vortex_2d"
    prob.pde = PDE_NAVIER_STOKES
    prob.ns = _ns_params(mu, viscosity=viscosity)
    return prob


def ns_periodic_field_2d(n: int = 4, p: int = 3, mu: float = 0.05, viscosity=VISCOSITY_CONSTANT) -> DGProblem:
    """Straight periodic QUAD box [0, 2 pi]^2 with a smooth non-uniform state (density, velocity and pressure
    waves); a test field for the viscous operator's consistency."""
    L = 2.0 * math.pi
    mesh = StructuredMesh(2, n, 0.0, L)
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops)
    prob = DGProblem("ns_periodic_field_2d", 2, PDE_NAVIER_STOKES, NUM_FLUX_ROE_PIKE, True, np.zeros(3), ops, mesh,
                     geom, sol=np.zeros((mesh.n_volumes, 4, ops.n_vs)), dt=0.0, n_steps=10,
                     ns=_ns_params(mu, viscosity=viscosity))
    x = prob.solution_node_xyz()
    prob.sol = _pack_state(ns_field_2d(x[..., 0], x[..., 1]))
    prob.dt = stable_dt(prob)
    return prob


def ns_field_2d(X, Y):
    """Conserved variables (4, ...) of the smooth periodic test field of ns_periodic_field_2d."""
    rho = 1.0 + 0.2 * np.sin(X) * np.cos(Y)
    vel = np.stack([0.3 + 0.2 * np.cos(X + Y), -0.1 + 0.15 * np.sin(2 * X - Y)])
    pr = 1.0 + 0.1 * np.cos(X) * np.sin(2 * Y)
    return primitive_to_conserved(2, rho, vel, pr)


def ns_channel(d: int = 2, n: int = 6, p: int = 3, mu: float = 0.01, mach: float = 0.3,
               num_flux: int = NUM_FLUX_ROE_PIKE, amplitude: float = 0.0, perturb: float = 0.1) -> DGProblem:
    """Navier-Stokes between no-slip adiabatic walls (BC_NOSLIP_ADIABATIC) at y = 0 and y = 2 pi, periodic in the
    other directions: rho = 1, p = 1 / (gamma Ma^2), u = sin(y / 2) (1 + perturb cos x), v = perturb sin x sin(y / 2)
    (zero on the walls), w = 0."""
    L = 2.0 * math.pi
    per = tuple(k != 1 for k in range(d))
    mesh = StructuredMesh(d, n, 0.0, L, periodic=per)
    ops = TPOperatorSet(mesh.e_type, p)
    deform = None
    if amplitude > 0:
        deform = sinusoidal_deform_2d(amplitude, L) if d == 2 else sinusoidal_deform_3d(amplitude, L)
    geom = TPGeometry(mesh, ops, deform=deform, curved=amplitude > 0)
    prob = DGProblem(f"ns_channel_{d}d", d, PDE_NAVIER_STOKES, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, d + 2, ops.n_vs)), dt=0.0, n_steps=100, ns=_ns_params(mu))
    x = prob.solution_node_xyz()
    X, Y = x[..., 0], x[..., 1]
    wall = np.sin(0.5 * Y)
    vel = [wall * (1.0 + perturb * np.cos(X)), perturb * np.sin(X) * wall] + ([np.zeros_like(X)] if d == 3 else [])
    pr = np.full_like(X, 1.0 / (GAMMA * mach * mach))
    prob.sol = _pack_state(primitive_to_conserved(d, np.ones_like(X), np.stack(vel), pr))
    prob.dt = stable_dt(prob)
    sides = {(1, 0): BC_NOSLIP_ADIABATIC, (1, 1): BC_NOSLIP_ADIABATIC}
    return _set_boundaries(prob, sides, _uniform_flow(d, 1.0, (0.0,) * d, 1.0 / (GAMMA * mach * mach)))


def ns_riemann_vortex_2d(n: int = 6, p: int = 3, mu: float = 0.01, num_flux: int = NUM_FLUX_ROE_PIKE) -> DGProblem:
    """euler_riemann_2d (the curved vortex box with characteristic boundaries on every side) with viscosity mu."""
    prob = euler_riemann_2d(n, p, num_flux=num_flux)
    prob.name = "ns_riemann_vortex_2d"
    prob.pde = PDE_NAVIER_STOKES
    prob.ns = _ns_params(mu)
    return prob


def annulus_deform(r_i: float, r_o: float):
    """Maps the unit square onto the annulus r_i <= r <= r_o: x -> r = r_i + (r_o - r_i) x, y -> theta = 2 pi y."""
    def f(x):
        r = r_i + (r_o - r_i) * x[:, 0]
        th = 2.0 * math.pi * x[:, 1]
        return np.stack([r * np.cos(th), r * np.sin(th)], axis=1)
    return f


def taylor_couette_state(x, y, r_i, r_o, omega, mu, Pr, r_s, t_b, p_b, dTdn):
    """The reference's Taylor-Couette solution (solution_taylor_couette_T.c:136-179, after Illingworth 1950):
    azimuthal velocity c (1/r - r/r_o^2), c = omega / (1/r_i^2 - 1/r_o^2), the temperature of the viscous heating
    with conductivity kappa = mu Cp / Pr and the outer wall's gradient dTdn, uniform pressure p_b, rho = p / (r_s T).
    Returns the conserved variables (4, ...)."""
    r, th = np.sqrt(x * x + y * y), np.arctan2(y, x)
    c = omega / (1.0 / r_i ** 2 - 1.0 / r_o ** 2)
    mu_kappa = Pr / (GAMMA / GM1 * r_s)                    # mu / kappa, kappa = mu Cp / Pr (also for mu = 0)
    vt = c * (1.0 / r - r / r_o ** 2)
    t = (t_b - 2.0 * c * c / r_o ** 2 * mu_kappa * np.log(r / r_i) - c * c * mu_kappa * (1.0 / r ** 2 - 1.0 / r_i ** 2)
         + dTdn * r_o * np.log(r / r_i))
    pr = np.full_like(r, p_b)
    return primitive_to_conserved(2, pr / (r_s * t), np.stack([-np.sin(th) * vt, np.cos(th) * vt]), pr)


def annulus_vertices(n, r_i: float = 0.5, r_o: float = 1.0, rotate: float = 0.0):
    """The straight QUAD mesh of the annulus r_i <= r <= r_o with n = n_r or (n_r, n_theta) volumes: volume (i, j) of
    StructuredMesh(2, (n_r, n_theta), 0, 1, periodic=(False, True)) has its vertices on the circles
    r_i + (r_o - r_i) (i + {0, 1}) / n_r at the angles 2 pi (j + {0, 1}) / n_theta + rotate. Returns xyz_ve
    (n_volumes, 2, 4) in the TP vertex order and face_curved (n_volumes, 4), 1 on the faces on r_i (local face 0)
    and r_o (local face 1), the reference's curved boundaries."""
    n_r, n_t = (n, n) if np.ndim(n) == 0 else (int(n[0]), int(n[1]))
    mesh = StructuredMesh(2, (n_r, n_t), 0.0, 1.0, periodic=(False, True))
    ve = np.empty((mesh.n_volumes, 2, 4))
    fc = np.zeros((mesh.n_volumes, 4), dtype=np.int32)
    for v in range(mesh.n_volumes):
        i, j = (int(k) for k in mesh.ijk[v][:2])
        for k in range(4):
            r = r_i + (r_o - r_i) * (i + (k & 1)) / n_r
            th = 2.0 * math.pi * (j + (k >> 1)) / n_t + rotate
            ve[v, :, k] = (r * math.cos(th), r * math.sin(th))
        fc[v, 0] = 1 if i == 0 else 0
        fc[v, 1] = 1 if i == n_r - 1 else 0
    return ve, fc


def ns_taylor_couette(n=8, p: int = 3, mu: float = 1e-3, omega: float = 1.0, diabatic: bool = False,
                      dTdn: float = 1.0, num_flux: int = NUM_FLUX_ROE_PIKE, perturb: float = 0.0,
                      geom_coef=None) -> DGProblem:
    """The reference's Navier-Stokes Taylor-Couette case (input_files/navier_stokes/steady/taylor_couette, mesh
    meshes/n-cylinder_hollow/2d.geo) on a curved QUAD annulus, n = n_r or (n_r, n_theta) volumes, r_i = 0.5,
    r_o = 1, periodic in theta:
    the inner cylinder rotates at omega (BC_NOSLIP_ALL_ROTATING with rho_b = 1, E_b = p_b / (gamma - 1) +
    rho_b (omega r_i)^2 / 2), the outer one is a static adiabatic wall (BC_NOSLIP_ADIABATIC), or a diabatic one
    with the normal temperature gradient dTdn (BC_NOSLIP_DIABATIC, solution_diabatic.data). Pr = 0.72, r_s = 1,
    p_b = t_b = 1; the state is the reference's Taylor-Couette solution, its density scaled by
    1 + perturb sin(3 theta) sin(pi (r - r_i) / (r_o - r_i)). The geometry is the exact polar map, or geom_coef
    ((n_volumes, (p+1)^2, 2) at the GLL nodes of order p, e.g. the blended geometry of annulus_vertices(n))."""
    r_i, r_o, Pr, r_s, p_b, t_b = 0.5, 1.0, 0.72, 1.0, 1.0, 1.0
    n_r, n_t = (n, n) if np.ndim(n) == 0 else (int(n[0]), int(n[1]))
    mesh = StructuredMesh(2, (n_r, n_t), 0.0, 1.0, periodic=(False, True))
    ops = TPOperatorSet(mesh.e_type, p)
    if geom_coef is None:
        geom = TPGeometry(mesh, ops, deform=annulus_deform(r_i, r_o), curved=True)
    else:
        geom = TPGeometry(mesh, ops, curved=True, coef=geom_coef)
    ns = _ns_params(mu, Pr=Pr, r_s=r_s)
    ns["dTdn"] = float(dTdn) if diabatic else 0.0
    prob = DGProblem("ns_taylor_couette", 2, PDE_NAVIER_STOKES, num_flux, True, np.zeros(3), ops, mesh, geom,
                     sol=np.zeros((mesh.n_volumes, 4, ops.n_vs)), dt=0.0, n_steps=100, ns=ns)
    x = prob.solution_node_xyz()
    X, Y = x[..., 0], x[..., 1]
    U = taylor_couette_state(X, Y, r_i, r_o, omega, mu, Pr, r_s, t_b, p_b, ns["dTdn"])
    if perturb:
        R, TH = np.sqrt(X * X + Y * Y), np.arctan2(Y, X)
        U = U * (1.0 + perturb * np.sin(3.0 * TH) * np.sin(math.pi * (R - r_i) / (r_o - r_i)))[None]
    prob.sol = _pack_state(U)
    prob.dt = stable_dt(prob, h=min((r_o - r_i) / n_r, 2.0 * math.pi * r_i / n_t))
    outer = BC_NOSLIP_DIABATIC if diabatic else BC_NOSLIP_ADIABATIC
    prob.meta.update(n=(n_r, n_t), p=p, omega=omega, r_i=r_i, r_o=r_o)
    return _set_boundaries(prob, {(0, 0): BC_NOSLIP_ALL_ROTATING, (0, 1): outer},
                           _taylor_couette_wall(r_i, omega, p_b))


def _taylor_couette_wall(r_i: float, omega: float, p_b: float, rho_b: float = 1.0):
    """The rotating wall's state (rho_b, rho_b u_wall, E_b) at face points xyz (m, 2): compute_uvw_ex_rotating
    (boundary_navier_stokes_T.c:507-523), the wall's velocity omega r e_theta; E_b = p_b / (gamma - 1) +
    rho_b (omega r_i)^2 / 2."""
    E_b = p_b / GM1 + 0.5 * rho_b * (omega * r_i) ** 2

    def wall_state(xyz):
        r, th = np.sqrt(xyz[:, 0] ** 2 + xyz[:, 1] ** 2), np.arctan2(xyz[:, 1], xyz[:, 0])
        vt = omega * r
        return np.stack([np.full(len(r), rho_b), -rho_b * np.sin(th) * vt, rho_b * np.cos(th) * vt,
                         np.full(len(r), E_b)], axis=1)
    return wall_state


def cylinder_parametric_map(xy):
    """The reference's map of its square annulus onto the circular annulus (constructor_xyz_cylinder_parametric_T,
    geometry_parametric_T.c:128-173): the radius is max(|x|, |y|) and the polar angle runs linearly along each side
    of the square, with the same branches on the angle of (x, y)."""
    x, y = xy[:, 0], xy[:, 1]
    r = np.maximum(np.abs(x), np.abs(y))
    t = np.arctan2(y, x)
    q = math.pi / 4.0
    out = np.full_like(t, np.nan)
    c0 = (t >= -q) & (t < q)
    c1 = (t >= q) & (t < 3.0 * q)
    c2 = ((t >= 3.0 * q) & (t <= 4.0 * q)) | ((t >= -4.0 * q) & (t < -3.0 * q))
    c3 = (t >= -3.0 * q) & (t < -q)
    out[c0] = y[c0] / r[c0] * q
    out[c1] = 0.5 * math.pi - x[c1] / r[c1] * q
    out[c2] = math.pi - y[c2] / r[c2] * q
    out[c3] = 1.5 * math.pi + x[c3] / r[c3] * q
    if np.any(np.isnan(out)):
        raise ValueError("point outside the map's branches")
    return np.stack([r * np.cos(out), r * np.sin(out)], axis=1)


def supersonic_vortex_state(x, y, r_i: float = 1.0, m_i: float = 2.25, rho_i: float = 1.0):
    """The reference's supersonic vortex (solution_supersonic_vortex_T.c:70-107, after Aftosmis et al. 1995):
    rho = rho_i (1 + (gamma - 1) / 2 m_i^2 (1 - (r_i / r)^2))^(1 / (gamma - 1)), p = rho^gamma, the azimuthal
    velocity r_i c_i m_i / r (c_i = sqrt(gamma) rho_i^((gamma - 1) / 2)) turning clockwise. Conserved (4, ...)."""
    r, t = np.sqrt(x * x + y * y), np.arctan2(y, x)
    c_i = math.sqrt(GAMMA) * rho_i ** (0.5 * GM1)
    vt = -r_i * c_i * m_i / r
    rho = rho_i * (1.0 + 0.5 * GM1 * m_i * m_i * (1.0 - (r_i / r) ** 2)) ** (1.0 / GM1)
    return primitive_to_conserved(2, rho, np.stack([-np.sin(t) * vt, np.cos(t) * vt]), rho ** GAMMA)


def euler_supersonic_vortex(path, p: int = 3, num_flux: int = NUM_FLUX_ROE_PIKE, perturb: float = 0.0):
    """The reference's steady/supersonic_vortex case on its own parametric domain: the quarter square annulus of the
    gmsh file `path` (gmsh.write_quarter_square_annulus_msh; r_i = 1, r_o = 1.384) mapped by cylinder_parametric_map
    the way the reference maps a parametric domain; m_i = 2.25, rho_i = 1. Riemann faces on the radial lines (their
    exterior state the exact solution), slip walls on the arcs; the state is the exact solution with its density
    scaled by 1 + perturb sin(4 theta) sin(pi (r - r_i) / (r_o - r_i))."""
    from .gmsh import gmsh_tp_problem
    r_i, r_o = 1.0, 1.384

    def exact(xy):
        return np.asarray(supersonic_vortex_state(xy[:, 0], xy[:, 1], r_i)).T

    def state(xy):
        U = exact(xy)
        if perturb:
            R, TH = np.sqrt(xy[:, 0] ** 2 + xy[:, 1] ** 2), np.arctan2(xy[:, 1], xy[:, 0])
            U = U * (1.0 + perturb * np.sin(4.0 * TH) * np.sin(math.pi * (R - r_i) / (r_o - r_i)))[:, None]
        return U
    prob = gmsh_tp_problem(path, 2, p, PDE_EULER, num_flux, state, exterior=exact,
                           parametric=cylinder_parametric_map, name="euler_supersonic_vortex")
    prob.meta.update(p=p, r_i=r_i, r_o=r_o)
    return prob


def ns_taylor_couette_parametric(path, p: int = 3, mu: float = 1e-3, omega: float = 1.0, diabatic: bool = False,
                                 dTdn: float = 1.0, num_flux: int = NUM_FLUX_ROE_PIKE, perturb: float = 0.0,
                                 viscosity: int = VISCOSITY_CONSTANT):
    """The reference's Taylor-Couette case on its own parametric domain: the square-annulus QUAD mesh of the gmsh
    file `path` (gmsh.write_square_annulus_msh, the PARAMETRIC domain of meshes/n-cylinder_hollow/2d.geo) mapped by
    cylinder_parametric_map the way the reference maps a parametric domain. Walls, constants and state as
    ns_taylor_couette (the state's density scaled by 1 + perturb sin(3 theta) sin(pi (r - r_i) / (r_o - r_i)));
    the BC codes come from the file (the outer wall's code sets adiabatic or diabatic); viscosity: constant mu or
    Sutherland's law scaled by mu."""
    from .gmsh import gmsh_tp_problem
    r_i, r_o, Pr, r_s, p_b, t_b = 0.5, 1.0, 0.72, 1.0, 1.0, 1.0
    ns = _ns_params(mu, Pr=Pr, r_s=r_s, viscosity=viscosity)
    ns["dTdn"] = float(dTdn) if diabatic else 0.0

    def state(xy):
        X, Y = xy[:, 0], xy[:, 1]
        U = taylor_couette_state(X, Y, r_i, r_o, omega, mu, Pr, r_s, t_b, p_b, ns["dTdn"])
        if perturb:
            R, TH = np.sqrt(X * X + Y * Y), np.arctan2(Y, X)
            U = U * (1.0 + perturb * np.sin(3.0 * TH) * np.sin(math.pi * (R - r_i) / (r_o - r_i)))[None]
        return np.asarray(U).T
    prob = gmsh_tp_problem(path, 2, p, PDE_NAVIER_STOKES, num_flux, state, exterior=_taylor_couette_wall(r_i, omega, p_b),
                           ns=ns, parametric=cylinder_parametric_map, name="ns_taylor_couette_parametric")
    prob.meta.update(p=p, omega=omega, r_i=r_i, r_o=r_o)
    return prob
