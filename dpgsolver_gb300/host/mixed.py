"""Seeded mixed-order TP problems: a structured periodic QUAD/HEX mesh whose volumes carry their own p.

This is the caller-side set-up of a p-adapted mesh. Volumes of the same p form one (element type, p) group with
its own TP operator set (the reference indexes its Solver_Element operators by p, element_solver.h:31-74).
Faces are integrated at the order p_f = max(p_L, p_R) (face_solver.c:123-132): their normals and Jacobians are
those of the side-0 volume at the GL(q_f) face nodes, as for uniform meshes (compute_geometry_face_T,
geometry_T.c:274-325). Geometry is isoparametric per volume (order p for curved volumes, 1 for straight ones,
geometry_T.c:740-742), so a curved mixed mesh is not watertight between volumes of different p, exactly as in
the reference; the straight mesh is.

State layout: one flat array, per volume the (n_var x n_vs(v)) block of the reference's column-major
(n_vs x n_var) sol_coef, concatenated in volume-list order.
"""
from __future__ import annotations

import math

import numpy as np

from .element import TPOperatorSet, gauss_lobatto, gauss_legendre, lagrange_matrix, kron_tp, tp_weights
from .geometry import TPGeometry, apply_nodes, sinusoidal_deform_2d, sinusoidal_deform_3d
from .mesh import StructuredMesh
from .problem import (BC_NOSLIP_ADIABATIC, BC_NOSLIP_ALL_ROTATING, BC_NOSLIP_DIABATIC, BC_RIEMANN, GAMMA, GM1,
                      NUM_FLUX_LAX_FRIEDRICHS, NUM_FLUX_ROE_PIKE, NUM_FLUX_UPWIND, PDE_ADVECTION, PDE_EULER,
                      PDE_NAVIER_STOKES, VISCOSITY_CONSTANT, VISCOSITY_SUTHERLAND, _ns_params, isentropic_vortex,
                      primitive_to_conserved)


class MixedTPProblem:
    """Mesh + per-volume p + per-group operators and geometry + state (flat, see the module docstring)."""

    def __init__(self, name, d, pde, num_flux, positivity, b_adv, mesh: StructuredMesh, p_vol, deform=None,
                 curved=False, parametric=None):
        self.name = name
        self.d = d
        self.pde = pde
        self.num_flux = num_flux
        self.positivity = bool(positivity)
        self.b_adv = np.asarray(b_adv, dtype=np.float64)
        self.mesh = mesh
        self.n_var = 1 if pde == PDE_ADVECTION else d + 2
        self.ns = None          # Navier-Stokes constants (viscosity model, mu, Pr, r_s, dTdn) when pde is 4
        p_vol = np.asarray(p_vol, dtype=np.int32)
        ps = sorted(set(int(p) for p in p_vol))
        self.groups = [TPOperatorSet(mesh.e_type, p) for p in ps]
        gidx = {p: g for g, p in enumerate(ps)}
        self.vol_group = np.array([gidx[int(p)] for p in p_vol], dtype=np.int32)
        self.p_vol = p_vol
        self.meta = {}
        nv = mesh.n_volumes
        # per-volume sizes and offsets
        q = np.array([self.groups[g].q for g in self.vol_group], dtype=np.int64)
        self.n_vs = q ** d
        self.state_off = np.zeros(nv + 1, dtype=np.int64)
        self.state_off[1:] = np.cumsum(self.n_var * self.n_vs)
        # geometry per group
        self.geoms = []
        self.group_vols = []
        from_file = getattr(mesh, "gmsh", None) is not None   # a QUAD/HEX mesh read from a file (GmshTPMesh)
        if from_file and (deform is not None or curved):
            raise ValueError("a mesh read from a file is taken straight (its vertices)")
        for g, ops in enumerate(self.groups):
            vols = np.nonzero(self.vol_group == g)[0]
            self.group_vols.append(vols)
            if not len(vols):
                self.geoms.append(None)
            elif from_file and parametric is not None:   # each group at its own geometry order (isoparametric)
                from .geometry import parametric_quad_coef
                self.geoms.append(TPGeometry(mesh, ops, curved=True, vols=vols,
                                             coef=parametric_quad_coef(mesh.vertices, ops.p, parametric)))
            elif from_file:
                self.geoms.append(TPGeometry(mesh, ops, curved=False, coef=mesh.vertices, vols=vols))
            else:
                self.geoms.append(TPGeometry(mesh, ops, deform=deform, curved=curved, vols=vols))
        self.curved = bool(curved) or parametric is not None
        self._face_geometry()
        self.sol = np.zeros(int(self.state_off[-1]))
        self.dt = 0.0
        self.bc = None          # (n_faces,) BC code per face (0 inside) when the mesh has boundary faces
        self.bc_state = None    # (face nodes, n_var): exterior state at every face node, face blocks in face order
        self.bc_data = None

    # ---- faces at p_f = max(p_L, p_R) ---------------------------------------------------------------------------
    def _face_geometry(self):
        mesh, d = self.mesh, self.d
        qv = np.array([self.groups[g].q for g in self.vol_group], dtype=np.int64)
        v1 = mesh.face_vol[:, 1]
        q1 = np.where(v1 >= 0, qv[np.maximum(v1, 0)], 0)          # a boundary face has side 0 only
        self.face_q = np.maximum(qv[mesh.face_vol[:, 0]], q1).astype(np.int32)
        n_fc = self.face_q.astype(np.int64) ** (d - 1)
        self.face_off = np.zeros(mesh.n_faces + 1, dtype=np.int64)
        self.face_off[1:] = np.cumsum(n_fc)
        nfn = int(self.face_off[-1])
        self.normals_fc = np.empty((nfn, d))
        self.jacobian_det_fc = np.empty(nfn)
        self.xyz_fc = np.empty((nfn, d))
        pos_in_group = np.empty(mesh.n_volumes, dtype=np.int64)
        for g, vols in enumerate(self.group_vols):
            pos_in_group[vols] = np.arange(len(vols))
        v0 = mesh.face_vol[:, 0]
        g0 = self.vol_group[v0]
        for lf in range(2 * d):
            nd = lf // 2
            val = np.array([-1.0 if lf % 2 == 0 else 1.0])
            for g, ops in enumerate(self.groups):
                geom = self.geoms[g]
                if geom is None:
                    continue
                for qf in np.unique(self.face_q):
                    sel = np.nonzero((mesh.face_lf[:, 0] == lf) & (g0 == g) & (self.face_q == qf))[0]
                    if len(sel) == 0:
                        continue
                    x_f, _ = gauss_legendre(int(qf))
                    one_d = [lagrange_matrix(geom.x_g, val) if k == nd else lagrange_matrix(geom.x_g, x_f)
                             for k in range(d)]
                    I_mf = kron_tp(one_d)
                    m_fc = apply_nodes(I_mf, geom.metrics_vm[pos_in_group[v0[sel]]])
                    nun = np.einsum("vnij,j->vni", m_fc, ops.normals_ref[lf])
                    nrm = np.sqrt(np.sum(nun * nun, axis=-1))
                    nff = int(qf) ** (d - 1)
                    rows = (self.face_off[sel][:, None] + np.arange(nff)[None, :]).ravel()
                    self.normals_fc[rows] = (nun / nrm[..., None]).reshape(-1, d)
                    self.jacobian_det_fc[rows] = nrm.ravel()
                    self.xyz_fc[rows] = apply_nodes(I_mf, geom.X_geom[pos_in_group[v0[sel]]]).reshape(-1, d)

    # ---- layout helpers -------------------------------------------------------------------------------------------
    @property
    def n_volumes(self) -> int:
        return self.mesh.n_volumes

    @property
    def n_state(self) -> int:
        return int(self.state_off[-1])

    def block(self, state, v):
        """(n_var, n_vs(v)) view of volume v's block of a flat state."""
        return state[self.state_off[v]:self.state_off[v + 1]].reshape(self.n_var, -1)

    def group_view(self, state, g):
        """(n_vols_g, n_var, n_vs_g) copy of group g's blocks (volume-list order within the group)."""
        vols = self.group_vols[g]
        n = self.n_var * self.groups[g].n_vs
        idx = self.state_off[vols][:, None] + np.arange(n)[None, :]
        return state[idx].reshape(len(vols), self.n_var, self.groups[g].n_vs)

    def set_group(self, state, g, blocks):
        vols = self.group_vols[g]
        n = self.n_var * self.groups[g].n_vs
        idx = self.state_off[vols][:, None] + np.arange(n)[None, :]
        state[idx] = np.asarray(blocks).reshape(len(vols), n)

    def solution_node_xyz(self, g):
        """Physical coordinates of group g's solution (GLL) nodes, (n_vols_g, n_vs_g, d)."""
        geom, ops = self.geoms[g], self.groups[g]
        L = kron_tp([lagrange_matrix(geom.x_g, ops.x_vs)] * self.d)
        return apply_nodes(L, geom.X_geom)

    def nc_fc(self) -> np.ndarray:
        """Right-trace gather permutation of every face at its order q_f, concatenated: the identity on an aligned
        structured mesh; on a mesh read from a file, the one its two sides' vertex correspondence gives
        (get_operator__nc_fc_T(1, face), compute_face_rlhs_T.c:133-146)."""
        if not self.mesh.n_faces:
            return np.zeros(0, np.int32)
        gm = getattr(self.mesh, "gmsh", None)
        if gm is None:
            return np.concatenate([np.arange(n, dtype=np.int32) for n in np.diff(self.face_off)])
        from .gmsh import tp_face_permutation
        out = []
        for f in range(self.mesh.n_faces):
            qf = int(self.face_q[f])
            if self.mesh.face_vol[f, 1] >= 0:
                out.append(np.asarray(tp_face_permutation(gm.face_match[f], qf, self.d), dtype=np.int32))
            else:
                out.append(np.arange(qf ** (self.d - 1), dtype=np.int32))
        return np.concatenate(out)

    def flat(self) -> dict:
        """The flat multi-group layout of the C ABIs (volume blocks in list order, face blocks in face order)."""
        nv, d = self.mesh.n_volumes, self.d
        mvc = [None] * nv
        jvc = [None] * nv
        for g, vols in enumerate(self.group_vols):
            if len(vols) == 0:
                continue
            geom = self.geoms[g]
            m = np.transpose(geom.metrics_vc, (0, 3, 2, 1))   # (v, j, i, n): column-major (n, i, j) per volume
            for k, v in enumerate(vols):
                mvc[v] = m[k].ravel()
                jvc[v] = geom.jacobian_det_vc[k]
        return {
            "groups": self.groups,
            "vol_group": self.vol_group,
            "face_q": self.face_q,
            "metrics_vc": np.concatenate(mvc),
            "jacobian_det_vc": np.concatenate(jvc),
            "normals_fc": np.ascontiguousarray(self.normals_fc).ravel(),
            "jacobian_det_fc": np.ascontiguousarray(self.jacobian_det_fc),
            "nc_fc": self.nc_fc(),
            "sol": self.sol,
            "bc_fc": None if self.bc is None else np.ascontiguousarray(self.bc, dtype=np.int32),
            "bc_state_fc": None if self.bc_state is None else np.ascontiguousarray(self.bc_state).ravel(),
            "bc_data": self.bc_data,
            "source_vc": getattr(self, "source_vc", None),
        }

    def set_boundaries(self, side_bc: dict | None, exterior):
        """BC code per boundary face from {(dim, side): code} (None: the codes of a mesh read from a file) and the
        exterior state exterior(xyz (m, d)) -> (m, n_var) at every face node (the test case's constructor_sol_bv);
        interior faces get code 0."""
        mesh = self.mesh
        self.bc = np.zeros(mesh.n_faces, dtype=np.int32)
        for f in np.nonzero(mesh.face_vol[:, 1] < 0)[0]:
            lf = int(mesh.face_lf[f, 0])
            self.bc[f] = mesh.face_bc[f] if side_bc is None else side_bc[(lf // 2, lf % 2)]
        ext = np.asarray(exterior(self.xyz_fc), dtype=np.float64).reshape(len(self.xyz_fc), self.n_var)
        inner = np.repeat(mesh.face_vol[:, 1] >= 0, np.diff(self.face_off))
        ext[inner] = 0.0
        self.bc_state = np.ascontiguousarray(ext)

    def stable_dt(self, cfl: float = 0.1) -> float:
        """dt = cfl * h / ((2 p_max + 1) * max(|V| + c)) over the solution nodes; with viscosity also the viscous
        bound of problem.stable_dt."""
        d = self.d
        lam, rho_min, T_max = 0.0, np.inf, 0.0
        for g in range(len(self.groups)):
            if len(self.group_vols[g]) == 0:
                continue
            U = self.group_view(self.sol, g)
            if self.pde != PDE_ADVECTION:
                rho = U[:, 0]
                vel = U[:, 1:1 + d] / rho[:, None]
                V2 = np.sum(vel * vel, axis=1)
                pr = GM1 * (U[:, d + 1] - 0.5 * rho * V2)
                lam = max(lam, float(np.max(np.sqrt(V2) + np.sqrt(GAMMA * pr / rho))))
                rho_min = min(rho_min, float(np.min(rho)))
                T_max = max(T_max, float(np.max(pr / rho)))
            else:
                lam = max(lam, float(np.linalg.norm(self.b_adv[:d])))
        h = float(np.min(self.mesh.h))
        k = 2 * max(g.p for g in self.groups) + 1
        dt = cfl * h / (k * lam)
        if self.ns is not None and self.ns["mu"] > 0.0:   # the viscous bound of problem.stable_dt
            mu = self.ns["mu"]
            if self.ns["viscosity"] == VISCOSITY_SUTHERLAND:
                mu *= 0.08 * math.sqrt(T_max / self.ns["r_s"])
            dt = min(dt, cfl * h * h / (k * k * GAMMA * mu / (self.ns["Pr"] * rho_min)))
        return dt


def _seeded_p(n_volumes, p_set, seed):
    rng = np.random.default_rng(seed)
    return rng.choice(np.asarray(p_set, dtype=np.int32), size=n_volumes)


def mixed_euler(d: int = 3, n: int = 58, p_set=(1, 2, 3, 4), num_flux: int = NUM_FLUX_ROE_PIKE, seed: int = 0,
                curved: bool = False, amplitude: float = 0.03, mach: float = 0.5, perturb: float = 0.05,
                positivity: bool = True, periodic=True, codes=None, mesh=None) -> MixedTPProblem:
    """Unit square/cube, per-volume p drawn uniformly from p_set (seeded), smooth seeded sinusoidal state
    around a free stream of Mach `mach`: rho = 1 + perturb * prod sin(2 pi x_k + phi_k), p = 1 + perturb * ...,
    velocity Mach * c along a fixed oblique direction with perturbations of the same form. periodic: per direction
    (all by default); codes: {(dim, side): BC code} for the ends of the other directions, whose exterior state is
    the unperturbed free stream. mesh: a QUAD/HEX mesh of the unit square/cube read from a file (gmsh.GmshTPMesh)
    instead of the structured one, e.g. with rotated local frames (its faces' nc_fc then permute)."""
    L = 1.0
    if mesh is None:
        mesh = StructuredMesh(d, n, 0.0, L, periodic=periodic)
    deform = None
    if curved:
        deform = sinusoidal_deform_2d(amplitude, L) if d == 2 else sinusoidal_deform_3d(amplitude, L)
    prob = MixedTPProblem("mixed_euler", d, PDE_EULER, num_flux, positivity, np.zeros(3), mesh,
                          _seeded_p(mesh.n_volumes, p_set, seed), deform=deform, curved=curved)
    rng = np.random.default_rng(seed + 1)
    ph = rng.uniform(0.0, 2.0 * math.pi, size=(d + 2, d))
    c0 = math.sqrt(GAMMA)
    dirn = np.array([1.0, 0.5, 0.25][:d])
    dirn /= np.linalg.norm(dirn)
    for g in range(len(prob.groups)):
        if len(prob.group_vols[g]) == 0:
            continue
        xyz = prob.solution_node_xyz(g)

        def wave(k):
            s = np.ones(xyz.shape[:2])
            for j in range(d):
                s = s * np.sin(2.0 * math.pi * xyz[..., j] / L + ph[k, j])
            return s
        rho = 1.0 + perturb * wave(0)
        pr = 1.0 + perturb * wave(1)
        vel = np.stack([mach * c0 * dirn[j] * (1.0 + perturb * wave(2 + j)) for j in range(d)])
        U = primitive_to_conserved(d, rho, vel, pr)          # (n_var, n_vols_g, n_vs)
        prob.set_group(prob.sol, g, np.transpose(U, (1, 0, 2)))
    prob.dt = prob.stable_dt()
    prob.meta.update(n=n, p_set=tuple(p_set), seed=seed, curved=curved)
    if np.any(mesh.face_vol[:, 1] < 0):
        vel0 = mach * c0 * dirn

        def stream(x):
            U = primitive_to_conserved(d, np.ones(len(x)), np.broadcast_to(vel0[:, None], (d, len(x))),
                                       np.ones(len(x)))
            return U.T
        prob.set_boundaries(codes, stream)
    return prob


def mixed_advection_2d(n: int = 8, p_set=(1, 2, 3, 4), seed: int = 0, b=(1.0, 0.5), curved: bool = False,
                       amplitude: float = 0.03, periodic=True, codes=None) -> MixedTPProblem:
    """[-1,1]^2, per-volume p from p_set (seeded), u0 = sin(pi x) sin(pi y), upwind flux; periodic per direction
    (all by default), codes {(dim, side): BC code} on the other ends with the exterior state u0 itself."""
    mesh = StructuredMesh(2, n, -1.0, 1.0, periodic=periodic)
    deform = sinusoidal_deform_2d(amplitude, 2.0) if curved else None
    prob = MixedTPProblem("mixed_advection_2d", 2, PDE_ADVECTION, NUM_FLUX_UPWIND, False,
                          np.array([b[0], b[1], 0.0]), mesh, _seeded_p(mesh.n_volumes, p_set, seed),
                          deform=deform, curved=curved)
    for g in range(len(prob.groups)):
        if len(prob.group_vols[g]) == 0:
            continue
        xyz = prob.solution_node_xyz(g)
        u = np.sin(math.pi * xyz[..., 0]) * np.sin(math.pi * xyz[..., 1])
        prob.set_group(prob.sol, g, u[:, None, :])
    prob.dt = prob.stable_dt()
    prob.meta.update(n=n, p_set=tuple(p_set), seed=seed, curved=curved)
    if np.any(mesh.face_vol[:, 1] < 0):
        prob.set_boundaries(codes, lambda x: (np.sin(math.pi * x[:, 0]) * np.sin(math.pi * x[:, 1]))[:, None])
    return prob


def mixed_vortex_2d(n: int = 8, p_set=(1, 2, 3, 4), seed: int = 0, num_flux: int = NUM_FLUX_ROE_PIKE,
                    curved: bool = True) -> MixedTPProblem:
    """Periodic [0,10]^2 with the isentropic vortex of strength 5 at (5,5) (as euler_vortex_2d), per-volume p."""
    L = 10.0
    mesh = StructuredMesh(2, n, 0.0, L)
    deform = sinusoidal_deform_2d(0.05, L) if curved else None
    prob = MixedTPProblem("mixed_vortex_2d", 2, PDE_EULER, num_flux, True, np.zeros(3), mesh,
                          _seeded_p(mesh.n_volumes, p_set, seed), deform=deform, curved=curved)
    for g in range(len(prob.groups)):
        if len(prob.group_vols[g]) == 0:
            continue
        xyz = prob.solution_node_xyz(g)
        rho, u, v, pr = isentropic_vortex(xyz, 5.0, 5.0, 5.0)
        U = primitive_to_conserved(2, rho, np.stack([u, v]), pr)
        prob.set_group(prob.sol, g, np.transpose(U, (1, 0, 2)))
    prob.dt = prob.stable_dt()
    prob.meta.update(n=n, p_set=tuple(p_set), seed=seed, curved=curved)
    return prob


def mixed_ns(d: int = 2, n: int = 6, p_set=(1, 2, 3, 4), num_flux: int = NUM_FLUX_ROE_PIKE, seed: int = 0,
             mu: float = 0.02, viscosity: int = VISCOSITY_CONSTANT, mach: float = 0.3, perturb: float = 0.1,
             curved: bool = False, amplitude: float = 0.03, walls=None, dTdn: float = 0.0) -> MixedTPProblem:
    """Navier-Stokes on [0, 2 pi]^d with per-volume p from p_set (seeded): rho = 1 + perturb sin x cos y,
    p = 1 / (gamma Ma^2), u = sin(y / 2) (1 + perturb cos x), v = perturb sin x sin(y / 2), w = perturb sin z
    (3D). walls: None (periodic) or {(1, side): BC code} for the ends y = 0 and y = 2 pi (no-slip adiabatic,
    diabatic with dTdn, rotating with the exterior state moving at u = 0.5, or Riemann with the unperturbed
    state outside); the other directions stay periodic."""
    L = 2.0 * math.pi
    per = True if walls is None else tuple(k != 1 for k in range(d))
    mesh = StructuredMesh(d, n, 0.0, L, periodic=per)
    deform = None
    if curved:
        deform = sinusoidal_deform_2d(amplitude, L) if d == 2 else sinusoidal_deform_3d(amplitude, L)
    prob = MixedTPProblem("mixed_ns", d, PDE_NAVIER_STOKES, num_flux, True, np.zeros(3), mesh,
                          _seeded_p(mesh.n_volumes, p_set, seed), deform=deform, curved=curved)
    prob.ns = dict(_ns_params(mu, viscosity=viscosity), dTdn=float(dTdn))
    p0 = 1.0 / (GAMMA * mach * mach)
    for g in range(len(prob.groups)):
        if len(prob.group_vols[g]) == 0:
            continue
        x = prob.solution_node_xyz(g)
        X, Y = x[..., 0], x[..., 1]
        wall = np.sin(0.5 * Y)
        vel = [wall * (1.0 + perturb * np.cos(X)), perturb * np.sin(X) * wall]
        if d == 3:
            vel.append(perturb * np.sin(x[..., 2]))
        rho = 1.0 + perturb * np.sin(X) * np.cos(Y)
        U = primitive_to_conserved(d, rho, np.stack(vel), np.full_like(X, p0))
        prob.set_group(prob.sol, g, np.transpose(U, (1, 0, 2)))
    prob.dt = prob.stable_dt()
    prob.meta.update(n=n, p_set=tuple(p_set), seed=seed, curved=curved, mu=mu)
    if walls is not None:
        def outside(xb):
            m = len(xb)
            u = np.zeros((d, m))
            rotating = any(c == BC_NOSLIP_ALL_ROTATING for c in walls.values())
            if rotating:
                u[0] = 0.5
            return primitive_to_conserved(d, np.ones(m), u, np.full(m, p0)).T
        prob.set_boundaries(walls, outside)
    return prob
