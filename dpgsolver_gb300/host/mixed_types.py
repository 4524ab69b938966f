"""Seeded conforming mixed-type 3D meshes (HEX, TET, WEDGE, PYR) with a p per volume (caller-side set-up).

The unit cube is divided into n^3 cells on a periodic grid, and each cell into volumes of one of three kinds:

* ``H``  one HEX;
* ``W``  two WEDGEs: the cell split by the diagonal plane through the diagonal (0,0)-(1,1) of its faces normal
  to the extrusion axis a (those two faces become two triangles each, the other four stay quads);
* ``C``  one pyramid or two tetrahedra per cell face, all sharing the cell centre as apex: a face that stays a
  quad carries a PYR (its base), a face split along the diagonal (0,0)-(1,1) of its tangential coordinates
  carries two TETs.

A cell face is a quad or two triangles the same way from both cells (the diagonal rule is translation invariant),
so the mesh is conforming; conflicting H/W neighbours are resolved by turning one of them into a C cell. All
volumes are affine images of the reference elements (dpgsolver_gb300.host.simplex), so metric terms and face
normals are constant per volume; a problem built with a ``deform`` (SineDeform) maps every volume through it
instead, and then they vary node by node (curved volumes). Cell kinds, wedge axes, the quad/triangle choice between
C cells and the p of every volume are drawn from seeded generators.

The face list follows the reference's rule (face.c:86-160): volumes are visited in list order and local faces in
index order, and the first volume met is side 0. Face nodes are laid out in one canonical vertex order per face:
the HEX side's own order when a HEX is on the face (so HEX volumes always see their faces unpermuted), else the
side-0 volume's order; face_ord[f, s] is the orientation index (simplex.TRI_ORDS / QUAD_ORDS) under which
side s sees that order.
"""
from __future__ import annotations

import math

import numpy as np

from .element import HEX, LINE, PYR, QUAD, TET, TRI, WEDGE, TPOperatorSet
from .problem import (GAMMA, GM1, NUM_FLUX_LAX_FRIEDRICHS, NUM_FLUX_ROE_PIKE, PDE_EULER,
                      primitive_to_conserved)
from . import simplex as S

_N_VERTS = {HEX: 8, TET: 4, WEDGE: 6, PYR: 5}


class MixedTypeMesh:
    """Volumes (type, global vertex ids, vertex coordinates) and faces with sides, local faces and orientations."""

    def __init__(self, n: int, seed: int = 0, c_blocks: float = 0.06, w_columns: float = 0.15,
                 p_tri: float = 1.0):
        """c_blocks: fraction of cells in 2x2x2 blocks of C cells; w_columns: fraction of the (i, j) columns made of
        W cells (extruded along z); p_tri: probability that a face between two C cells is split into triangles.
        The defaults give about 50 % HEX, 25 % TET, 15 % WEDGE and 10 % PYR volumes."""
        if n % 2:
            raise ValueError("n must be even (2x2x2 blocks)")
        self.n = n
        self.h = 1.0 / n
        rng = np.random.default_rng(seed)
        nc = n ** 3
        idx = np.arange(nc)
        ijk = np.stack([idx % n, (idx // n) % n, idx // (n * n)], axis=1)
        kind = np.zeros(nc, dtype=np.int64)                       # 0 H, 1 W, 2 C
        axis = np.full(nc, 2, dtype=np.int64)
        col = rng.random((n, n)) < w_columns
        kind[col[ijk[:, 0], ijk[:, 1]]] = 1
        nb = n // 2
        blk = rng.random((nb, nb, nb)) < c_blocks
        kind[blk[ijk[:, 0] // 2, ijk[:, 1] // 2, ijk[:, 2] // 2]] = 2

        def shifted(a, step):
            s = ijk.copy()
            s[:, a] = (s[:, a] + step) % n
            return s[:, 0] + n * (s[:, 1] + n * s[:, 2])

        nb_hi = [shifted(a, 1) for a in range(3)]
        nb_lo = [shifted(a, -1) for a in range(3)]

        def need(a):
            """Requirement of every cell on its faces normal to axis a: 0 quad, 1 two triangles, -1 none (C)."""
            return np.where(kind == 0, 0, np.where(kind == 1, (axis == a).astype(np.int64), -1))

        # resolve H/W conflicts by turning one side into a C cell (none arise with z-columns of W cells)
        while True:
            bad = False
            for a in range(3):
                r = need(a)
                r1, r2 = r, r[nb_hi[a]]
                clash = np.nonzero((r1 >= 0) & (r2 >= 0) & (r1 != r2))[0]
                if len(clash):
                    bad = True
                    flip = rng.random(len(clash)) < 0.5
                    kind[np.where(flip, nb_hi[a][clash], clash)] = 2
            if not bad:
                break
        # face kind between every cell and its +a neighbour: 1 = two triangles, 0 = quad
        fk = []
        for a in range(3):
            r = need(a)
            r1, r2 = r, r[nb_hi[a]]
            free = rng.random(nc) < p_tri
            fk.append(np.where(r1 >= 0, r1, np.where(r2 >= 0, r2, free.astype(np.int64))))
        self.cell_kind = kind

        # ---- volumes (coordinates in units of h/2: corners even, centres odd) ----
        V = n ** 3   # global vertex ids: corners i + n j + n^2 k (periodic), centres V + cell
        types, gids, units = [], [], []
        kl, il = kind.tolist(), ijk.tolist()
        fkl = [f.tolist() for f in fk]
        nbl = [x.tolist() for x in nb_lo]

        def corner(i, j, k):
            return (i % n) + n * ((j % n) + n * (k % n)), (2 * i, 2 * j, 2 * k)

        def face_corners(i, j, k, a, side):
            """The 4 corners of the cell face normal to a at side 0/1, tensor order in the tangential axes."""
            t0, t1 = [x for x in range(3) if x != a]
            out = []
            for dv in (0, 1):
                for du in (0, 1):
                    off = [0, 0, 0]
                    off[a] = side
                    off[t0] = du
                    off[t1] = dv
                    out.append(corner(i + off[0], j + off[1], k + off[2]))
            return out

        def add(t, verts):
            types.append(t)
            gids.append([v[0] for v in verts])
            units.append([v[1] for v in verts])

        for c in range(nc):
            i, j, k = il[c]
            if kl[c] == 0:
                add(HEX, [corner(i + dx, j + dy, k + dz) for dz in (0, 1) for dy in (0, 1) for dx in (0, 1)])
            elif kl[c] == 1:
                lo, hi = face_corners(i, j, k, 2, 0), face_corners(i, j, k, 2, 1)
                for tri in ((0, 1, 3), (0, 3, 2)):     # triangles of the diagonal (0,0)-(1,1)
                    add(WEDGE, [lo[m] for m in tri] + [hi[m] for m in tri])
            else:
                centre = (V + c, (2 * i + 1, 2 * j + 1, 2 * k + 1))
                for a in range(3):
                    for side in (0, 1):
                        tri_face = fkl[a][c] if side == 1 else fkl[a][nbl[a][c]]
                        fc = face_corners(i, j, k, a, side)
                        if not tri_face:
                            add(PYR, fc + [centre])
                        else:
                            for tri in ((0, 1, 3), (0, 3, 2)):
                                add(TET, [fc[m] for m in tri] + [centre])
        self.types = np.array(types, dtype=np.int32)
        self.n_volumes = len(types)
        # affine maps per type (batched), mirrored to a positive orientation where needed
        self.A = np.empty((self.n_volumes, 3, 3))
        self.b = np.empty((self.n_volumes, 3))
        self.X = [None] * self.n_volumes
        mirror = {TET: [0, 2, 1, 3], WEDGE: [0, 2, 1, 3, 5, 4], PYR: [0, 2, 1, 3, 4], HEX: [0, 2, 1, 3, 4, 6, 5, 7]}
        for t in (HEX, TET, WEDGE, PYR):
            sel = np.nonzero(self.types == t)[0]
            if len(sel) == 0:
                continue
            X = np.array([units[v] for v in sel], dtype=np.float64) * (0.5 * self.h)
            A, b0 = _affine_batch(t, X)
            neg = np.nonzero(np.linalg.det(A) < 0.0)[0]
            if len(neg):
                X[neg] = X[neg][:, mirror[t]]
                for r in neg:
                    g = gids[sel[r]]
                    gids[sel[r]] = [g[m] for m in mirror[t]]
                A[neg], b0[neg] = _affine_batch(t, X[neg])
            self.A[sel], self.b[sel] = A, b0
            for r, v in enumerate(sel):
                self.X[v] = X[r]
        self.gids = gids
        self._faces()

    def _faces(self):
        """Face list by the reference's rule, with canonical node order and per-side orientations."""
        seen = {}
        fv, flf = [], []
        for v in range(self.n_volumes):
            t = self.types[v]
            for lf, fve in enumerate(S.F_VE[t]):
                key = tuple(sorted(self.gids[v][m] for m in fve))
                if key in seen:
                    f = seen.pop(key)
                    fv[f][1], flf[f][1] = v, lf
                else:
                    seen[key] = len(fv)
                    fv.append([v, -1])
                    flf.append([lf, -1])
        if seen and getattr(self, "periodic", True):
            raise AssertionError("unmatched faces: the mesh is not conforming/periodic")
        self.face_vol = np.array(fv, dtype=np.int32)
        self.face_lf = np.array(flf, dtype=np.int32)
        self.n_faces = len(fv)
        self.face_ord = np.zeros((self.n_faces, 2), dtype=np.int32)
        self.face_canon = np.zeros(self.n_faces, dtype=np.int32)    # side whose local order is canonical
        tp = getattr(self, "tp_type", HEX)
        for f in range(self.n_faces):
            vs = self.face_vol[f]
            if vs[1] < 0:     # boundary face: side 0 only, in its own order
                continue
            cs = 1 if (self.types[vs[1]] == tp and self.types[vs[0]] != tp) else 0
            self.face_canon[f] = cs
            canon = [self.gids[vs[cs]][m] for m in S.F_VE[self.types[vs[cs]]][self.face_lf[f, cs]]]
            ft = {2: LINE, 3: S.TRI, 4: S.QUAD}[len(canon)]
            for s in range(2):
                loc = [self.gids[vs[s]][m] for m in S.F_VE[self.types[vs[s]]][self.face_lf[f, s]]]
                perm = tuple(loc.index(g) for g in canon)
                ords = S.face_ords(ft)
                if perm not in ords:
                    raise AssertionError("face orientation outside the symmetry group")
                self.face_ord[f, s] = ords.index(perm)

    def counts(self):
        return {int(t): int(np.sum(self.types == t)) for t in (HEX, TET, WEDGE, PYR)}


def _tp_face_points(d: int, lf: int, q: int) -> np.ndarray:
    """GL face nodes of local face lf of the reference QUAD/HEX (tangential coordinates in TP order)."""
    from .element import gauss_legendre
    x1, _ = gauss_legendre(q)
    nd, val = lf // 2, (-1.0 if lf % 2 == 0 else 1.0)
    tang = [k for k in range(d) if k != nd]
    if d == 2:
        pts = np.zeros((q, 2))
        pts[:, tang[0]] = x1
    else:
        pts = np.zeros((q * q, 3))
        pts[:, tang[0]] = np.tile(x1, q)
        pts[:, tang[1]] = np.repeat(x1, q)
    pts[:, nd] = val
    return pts


_AFF_SUB = {TET: [0, 1, 2, 3], WEDGE: [0, 1, 2, 3], PYR: [0, 1, 2, 4], HEX: [0, 1, 2, 4], TRI: [0, 1, 2],
            QUAD: [0, 1, 2]}


class MixedTriQuadMesh(MixedTypeMesh):
    """The 2D counterpart: the periodic unit square in n^2 cells, each (seeded, probability p_tri) one QUAD or two
    TRIs split along the diagonal (0,0)-(1,1) of the cell, both counter-clockwise. Conforming by construction; faces
    (edges) follow the same rule as the 3D mesh: the QUAD's own order when a QUAD is on the face, else side 0's,
    and face_ord indexes simplex.LINE_ORDS."""

    tp_type = QUAD

    def __init__(self, n: int, seed: int = 0, p_tri: float = 0.5, periodic: bool = True):
        if n < 2:
            raise ValueError("n >= 2")
        self.d, self.n = 2, n
        self.h = 1.0 / n
        self.periodic = bool(periodic)
        rng = np.random.default_rng(seed)
        types, gids, X = [], [], []

        def vid(i, j):
            if not periodic:   # the sides of the square are boundary faces
                return i + (n + 1) * j
            return (i % n) + n * (j % n)
        for j in range(n):
            for i in range(n):
                c = [(i, j), (i + 1, j), (i, j + 1), (i + 1, j + 1)]     # TP corner order
                if rng.random() < p_tri:
                    for tri in ((0, 1, 3), (0, 3, 2)):
                        types.append(TRI)
                        gids.append([vid(*c[m]) for m in tri])
                        X.append([c[m] for m in tri])
                else:
                    types.append(QUAD)
                    gids.append([vid(*cc) for cc in c])
                    X.append(c)
        self.types = np.array(types, dtype=np.int32)
        self.n_volumes = len(types)
        self.gids = gids
        self.A = np.empty((self.n_volumes, 2, 2))
        self.b = np.empty((self.n_volumes, 2))
        self.X = [np.asarray(x, dtype=np.float64) * self.h for x in X]
        for t in (QUAD, TRI):
            sel = np.nonzero(self.types == t)[0]
            if len(sel) == 0:
                continue
            A, b0 = _affine_batch(t, np.array([self.X[v] for v in sel]))
            self.A[sel], self.b[sel] = A, b0
        self._faces()

    def counts(self):
        return {int(t): int(np.sum(self.types == t)) for t in (QUAD, TRI)}


def _affine_batch(t, X):
    """A (n, 3, 3), b (n, 3) with X[:, m] = A r_m + b for the reference vertices r_m of type t (checked on every
    vertex: the volumes must be affine images of the reference element)."""
    R = S.VERTS[t]
    sub = _AFF_SUB[t]
    Rd = (R[sub[1:]] - R[sub[0]]).T                      # columns r_m - r_0
    Xd = np.transpose(X[:, sub[1:]] - X[:, [sub[0]]], (0, 2, 1))
    A = Xd @ np.linalg.inv(Rd)
    b = X[:, sub[0]] - A @ R[sub[0]]
    err = np.max(np.abs(np.einsum("vij,mj->vmi", A, R) + b[:, None, :] - X)) if len(X) else 0.0
    if err > 1e-12 * max(1.0, float(np.max(np.abs(X))) if len(X) else 1.0):
        raise AssertionError("volume is not an affine image of its reference element")
    return A, b


def _affine(t, x):
    """A, b with x_m = A r_m + b for the reference vertices r_m (affine volumes)."""
    R = S.VERTS[t]
    M, *_ = np.linalg.lstsq(np.hstack([R, np.ones((len(R), 1))]), x, rcond=None)
    A, b = M[:3].T, M[3]
    if np.max(np.abs(R @ A.T + b - x)) > 1e-12 * max(1.0, np.max(np.abs(x))):
        raise AssertionError("volume is not an affine image of its reference element")
    return A, b


class SineDeform:
    """x -> x + a prod_j sin(2 pi x_j) on every coordinate: a smooth map of the unit square / cube onto itself that
    is periodic and fixes its boundary, so a mesh of it stays conforming, periodic and bounded by the same faces."""

    def __init__(self, d: int, amplitude: float):
        self.d, self.a = d, float(amplitude)

    def __call__(self, x):
        s = np.prod(np.sin(2.0 * math.pi * x), axis=-1)
        return x + self.a * s[..., None]

    def jac(self, x):
        """dx'/dx at x (..., d) -> (..., d, d)."""
        sn, cs = np.sin(2.0 * math.pi * x), np.cos(2.0 * math.pi * x)
        g = np.empty_like(x)
        for j in range(self.d):
            g[..., j] = 2.0 * math.pi * cs[..., j] * np.prod(np.delete(sn, j, axis=-1), axis=-1)
        return np.eye(self.d) + self.a * g[..., None, :]


class MixedTypeProblem:
    """Mixed-type mesh + per-volume p + per-(type, p) operators + geometry + state (flat layout as MixedTPProblem:
    per volume the (n_var x n_vs(v)) block, volume-list order). Affine geometry, or with ``deform`` every volume's
    map composed with it: x(r) = deform(A r + b), whose metric terms m = J (dx/dr)^-T and Jacobian J are then taken
    at every cubature node, and the face normals and J_f at every face node (side 0's map)."""

    def __init__(self, mesh: MixedTypeMesh, p_vol, pde=PDE_EULER, num_flux=NUM_FLUX_ROE_PIKE, positivity=False,
                 deform=None):
        self.mesh = mesh
        self.d = d = getattr(mesh, "d", 3)
        tp = QUAD if d == 2 else HEX
        self.pde = pde
        self.num_flux = num_flux
        self.positivity = bool(positivity)
        self.b_adv = np.zeros(3)
        self.n_var = d + 2
        self.name = "mixed_types"
        self.meta = {}
        p_vol = np.asarray(p_vol, dtype=np.int32)
        keys = sorted(set((int(t), int(p)) for t, p in zip(mesh.types, p_vol)), key=lambda k: (k[0] != tp, k))
        self.groups = [TPOperatorSet(tp, p) if t == tp else S.DenseOperatorSet(t, p) for t, p in keys]
        self.group_key = keys
        gidx = {k: g for g, k in enumerate(keys)}
        self.vol_group = np.array([gidx[(int(t), int(p))] for t, p in zip(mesh.types, p_vol)], dtype=np.int32)
        self.p_vol = p_vol
        nv = mesh.n_volumes
        n_vs = np.array([self.groups[g].n_vs for g in self.vol_group], dtype=np.int64)
        self.n_vs = n_vs
        self.state_off = np.zeros(nv + 1, dtype=np.int64)
        self.state_off[1:] = np.cumsum(self.n_var * n_vs)
        self.group_vols = [np.nonzero(self.vol_group == g)[0] for g in range(len(self.groups))]
        # affine geometry per volume: m = J A^-T (m(n,i,j) = J dr_j/dx_i), J = det A
        self.A, self.b = mesh.A, mesh.b
        self.J = np.linalg.det(self.A)
        if np.any(self.J <= 0.0):
            raise AssertionError("non-positive Jacobian")
        self.m = self.J[:, None, None] * np.transpose(np.linalg.inv(self.A), (0, 2, 1))
        self.deform = deform
        if deform is not None:
            # per group (n_vols_g, n_vc, d, d) metric terms and (n_vols_g, n_vc) Jacobians at the cubature nodes
            self.m_vc, self.J_vc = [], []
            for g in range(len(self.groups)):
                m, J = self._map_metrics(self.group_vols[g], self._vc_ref(g))
                self.m_vc.append(m)
                self.J_vc.append(J)
        # faces at p_f = max(p_L, p_R), integrated as the reference does: q_f GL nodes on lines, q_f^2 on quads,
        # the Witherden-Vincent rule of degree 2 p_f on triangles
        q = p_vol.astype(np.int64) + 1
        self.face_q = np.maximum(q[mesh.face_vol[:, 0]], q[mesh.face_vol[:, 1]]).astype(np.int32)
        self.face_nvert = self._face_vertex_counts()
        n_fc = np.empty(mesh.n_faces, dtype=np.int64)
        for nvert, ft in ((2, LINE), (3, S.TRI), (4, S.QUAD)):
            for qf in np.unique(self.face_q):
                sel = (self.face_nvert == nvert) & (self.face_q == qf)
                if np.any(sel):
                    n_fc[sel] = len(S.face_rule(ft, int(qf))[1])
        self.face_off = np.zeros(mesh.n_faces + 1, dtype=np.int64)
        self.face_off[1:] = np.cumsum(n_fc)
        self._face_geometry()
        self.sol = np.zeros(int(self.state_off[-1]))
        self.dt = 0.0
        self.bc = None
        self.bc_state = None
        self.bc_data = None

    def _vc_ref(self, g):
        ops = self.groups[g]
        if getattr(ops, "dense", False):
            return ops.x_vc
        from .element import tp_nodes
        return tp_nodes(ops.x_vc, self.d)

    def _map(self, vols, xr):
        """Physical points (len(vols), n, d) of reference points xr (n, d), or (len(vols), n, d) per volume."""
        if xr.ndim == 2:
            y = np.einsum("vij,nj->vni", self.A[vols], xr) + self.b[vols][:, None, :]
        else:
            y = np.einsum("vij,vnj->vni", self.A[vols], xr) + self.b[vols][:, None, :]
        return y if self.deform is None else self.deform(y)

    def _map_metrics(self, vols, xr):
        """(m, J) at reference points xr of the volumes: dx/dr = D deform(A r + b) A, J = det, m = J (dx/dr)^-T
        (m(n, i, j) = J dr_j / dx_i, the reference's metrics_vc)."""
        if xr.ndim == 2:
            y = np.einsum("vij,nj->vni", self.A[vols], xr) + self.b[vols][:, None, :]
        else:
            y = np.einsum("vij,vnj->vni", self.A[vols], xr) + self.b[vols][:, None, :]
        F = self.deform.jac(y) @ self.A[vols][:, None, :, :]
        J = np.linalg.det(F)
        if np.any(J <= 0.0):
            raise AssertionError("non-positive Jacobian")
        return J[..., None, None] * np.swapaxes(np.linalg.inv(F), -1, -2), J

    def set_boundaries(self, code: int, exterior=None):
        """Every boundary face (face_vol[f, 1] < 0) gets the reference's BC code `code`; exterior(xyz (m, d)) ->
        (m, n_var) is the exterior state at their face nodes (the test case's constructor_sol_bv; zero when None, as
        slip walls need none)."""
        mesh = self.mesh
        bnd = mesh.face_vol[:, 1] < 0
        self.bc = np.where(bnd, int(code), 0).astype(np.int32)
        nfn = int(self.face_off[-1])
        ext = np.zeros((nfn, self.n_var))
        if exterior is not None:
            ext = np.asarray(exterior(self.face_xyz()), dtype=np.float64).reshape(nfn, self.n_var)
            ext[np.repeat(~bnd, np.diff(self.face_off))] = 0.0
        self.bc_state = np.ascontiguousarray(ext)

    def face_xyz(self):
        """Physical coordinates of every face's canonical nodes (side 0's map), (n_face_nodes, d)."""
        mesh = self.mesh
        out = np.empty((int(self.face_off[-1]), self.d))
        for f in range(mesh.n_faces):
            v, lf = int(mesh.face_vol[f, 0]), int(mesh.face_lf[f, 0])
            g = self.groups[self.vol_group[v]]
            qf = int(self.face_q[f])
            if getattr(g, "dense", False):
                xr = g.face_points(lf, int(mesh.face_ord[f, 0]), qf)
            else:
                xr = _tp_face_points(self.d, lf, qf)
            out[self.face_off[f]:self.face_off[f + 1]] = self._map(np.array([v]), xr)[0]
        return out

    def _face_vertex_counts(self):
        """Vertices of every face (2: LINE, 3: TRI, 4: QUAD), from its side-0 volume's local face."""
        mesh, d = self.mesh, self.d
        v0, lf0 = mesh.face_vol[:, 0], mesh.face_lf[:, 0]
        ftype = np.zeros(mesh.n_faces, dtype=np.int32)
        for t in ((QUAD, TRI) if d == 2 else (HEX, TET, WEDGE, PYR)):
            sel = np.nonzero(mesh.types[v0] == t)[0]
            if len(sel):
                ftype[sel] = np.array([len(fv) for fv in S.F_VE[t]])[lf0[sel]]
        return ftype

    def _face_geometry(self):
        """Normals and J_f of the side-0 volume (constant on affine faces) and the side-0 face-rule weights, at the
        canonical nodes of every face."""
        mesh, d = self.mesh, self.d
        v0, lf0 = mesh.face_vol[:, 0], mesh.face_lf[:, 0]
        nref = np.zeros((mesh.n_faces, d))
        ftype = self.face_nvert
        for t in ((QUAD, TRI) if d == 2 else (HEX, TET, WEDGE, PYR)):
            sel = np.nonzero(mesh.types[v0] == t)[0]
            if len(sel) == 0:
                continue
            if t in (HEX, QUAD):
                nr = TPOperatorSet(t, 1).normals_ref
            else:
                nr = S.reference_normals_2d(t) if d == 2 else S.reference_normals_3d(t)
            nref[sel] = nr[lf0[sel]]
        nfc = np.diff(self.face_off)
        if self.deform is None:
            nun = np.einsum("fij,fj->fi", self.m[v0], nref)
            jn = np.linalg.norm(nun, axis=1)
            self.normals_fc = np.repeat(nun / jn[:, None], nfc, axis=0)
            self.jacobian_det_fc = np.repeat(jn, nfc)
        else:
            # per face node: side 0's metric terms there applied to the reference normal of its local face
            self.normals_fc = np.empty((int(self.face_off[-1]), d))
            self.jacobian_det_fc = np.empty(int(self.face_off[-1]))
            o0 = mesh.face_ord[:, 0] if getattr(mesh, "face_ord", None) is not None else np.zeros(mesh.n_faces, int)
            keys = np.stack([self.vol_group[v0], lf0, o0, self.face_q], axis=1)
            for key in np.unique(keys, axis=0):
                g, lf, o, qf = (int(k) for k in key)
                sel = np.nonzero(np.all(keys == key, axis=1))[0]
                ops = self.groups[g]
                xr = ops.face_points(lf, o, qf) if getattr(ops, "dense", False) else _tp_face_points(d, lf, qf)
                m, _ = self._map_metrics(v0[sel], xr)                       # (n_sel, n_fc, d, d)
                nun = np.einsum("fnij,fj->fni", m, nref[sel])
                jn = np.linalg.norm(nun, axis=2)
                idx = (self.face_off[sel][:, None] + np.arange(len(xr))[None, :]).ravel()
                self.normals_fc[idx] = (nun / jn[..., None]).reshape(-1, d)
                self.jacobian_det_fc[idx] = jn.ravel()
        self.w_fc = np.empty(int(self.face_off[-1]))
        for nvert, ft in ((2, LINE), (3, S.TRI), (4, S.QUAD)):
            for qf in np.unique(self.face_q):
                sel = np.nonzero((ftype == nvert) & (self.face_q == qf))[0]
                if len(sel) == 0:
                    continue
                wr = S.face_rule(ft, int(qf))[1]
                idx = (self.face_off[sel][:, None] + np.arange(len(wr))[None, :]).ravel()
                self.w_fc[idx] = np.tile(wr, len(sel))

    # ---- layout helpers (as MixedTPProblem) ----
    @property
    def n_volumes(self) -> int:
        return self.mesh.n_volumes

    @property
    def n_state(self) -> int:
        return int(self.state_off[-1])

    def block(self, state, v):
        return state[self.state_off[v]:self.state_off[v + 1]].reshape(self.n_var, -1)

    def group_view(self, state, g):
        vols = self.group_vols[g]
        n = self.n_var * self.groups[g].n_vs
        idx = self.state_off[vols][:, None] + np.arange(n)[None, :]
        return state[idx].reshape(len(vols), self.n_var, self.groups[g].n_vs)

    def set_group(self, state, g, blocks):
        vols = self.group_vols[g]
        n = self.n_var * self.groups[g].n_vs
        idx = self.state_off[vols][:, None] + np.arange(n)[None, :]
        state[idx] = np.asarray(blocks).reshape(len(vols), n)

    def vc_xyz(self, g):
        """Physical coordinates of group g's volume cubature nodes (n_vols_g, n_vc, d)."""
        ops = self.groups[g]
        vols = self.group_vols[g]
        return self._map(vols, self._vc_ref(g))

    def nc_fc(self) -> np.ndarray:
        return np.concatenate([np.arange(n, dtype=np.int32) for n in np.diff(self.face_off)])

    def flat(self) -> dict:
        n_vc = np.array([self.groups[g].n_vc for g in self.vol_group], dtype=np.int64)
        vc_off = np.zeros(len(n_vc) + 1, dtype=np.int64)
        vc_off[1:] = np.cumsum(n_vc)
        dd = self.d * self.d
        mflat = np.empty(int(vc_off[-1]) * dd)
        jflat = np.empty(int(vc_off[-1]))
        for g, vols in enumerate(self.group_vols):
            if len(vols) == 0:
                continue
            nq = self.groups[g].n_vc
            idx = (dd * vc_off[vols])[:, None] + np.arange(dd * nq)[None, :]
            jidx = vc_off[vols][:, None] + np.arange(nq)[None, :]
            if self.deform is None:
                mt = np.transpose(self.m[vols], (0, 2, 1)).reshape(len(vols), dd)     # [j][i] per volume
                mflat[idx] = np.repeat(mt[:, :, None], nq, axis=2).reshape(len(vols), dd * nq)
                jflat[jidx] = np.repeat(self.J[vols][:, None], nq, axis=1)
            else:   # (n, i, j) at n + n_vc (i + d j)
                mflat[idx] = np.transpose(self.m_vc[g], (0, 3, 2, 1)).reshape(len(vols), dd * nq)
                jflat[jidx] = self.J_vc[g]
        mvc, jvc = [mflat], [jflat]
        return {
            "groups": self.groups,
            "vol_group": self.vol_group,
            "face_q": self.face_q,
            "face_ord": self.mesh.face_ord,
            "metrics_vc": np.concatenate(mvc),
            "jacobian_det_vc": np.concatenate(jvc),
            "normals_fc": np.ascontiguousarray(self.normals_fc).ravel(),
            "jacobian_det_fc": self.jacobian_det_fc.copy(),
            "nc_fc": self.nc_fc(),
            "sol": self.sol,
            "bc_fc": None if self.bc is None else np.ascontiguousarray(self.bc, dtype=np.int32),
            "bc_state_fc": None if self.bc_state is None else np.ascontiguousarray(self.bc_state).ravel(),
            "bc_data": self.bc_data,
            "source_vc": getattr(self, "source_vc", None),
        }

    def project(self, fn):
        """Set the state to the L2 projection of fn(xyz (m, 3)) -> (m, n_var) onto every volume's basis (volume
        cubature; HEX groups: values at the GLL solution nodes, which are their coefficients)."""
        from .element import tp_nodes
        for g, ops in enumerate(self.groups):
            vols = self.group_vols[g]
            if len(vols) == 0:
                continue
            if getattr(ops, "dense", False):
                x = self.vc_xyz(g)
                U = fn(x.reshape(-1, self.d)).reshape(len(vols), ops.n_vc, self.n_var)
                if self.deform is None:
                    # affine volume: coef = M_ref^-1 cv0^T diag(w) U
                    Pm = np.linalg.inv(ops.mass()) @ (ops.cv0_vs_vc().T * ops.w_vc[None, :])   # (n_vs, n_vc)
                    coef = np.transpose(U, (0, 2, 1)) @ Pm.T                                   # (v, k, a)
                else:
                    # curved volume: coef = M^-1 cv0^T diag(w J) U, M = cv0^T diag(w J) cv0
                    cv0 = ops.cv0_vs_vc()
                    wJ = ops.w_vc[None, :] * self.J_vc[g]                                     # (v, n)
                    M = np.einsum("na,vn,nb->vab", cv0, wJ, cv0)
                    rhs = np.einsum("na,vn,vnk->vak", cv0, wJ, U)
                    coef = np.transpose(np.linalg.solve(M, rhs), (0, 2, 1))
            else:
                xs = tp_nodes(ops.x_vs, self.d)
                x = self._map(vols, xs)
                coef = np.transpose(fn(x.reshape(-1, self.d)).reshape(len(vols), ops.n_vs, self.n_var), (0, 2, 1))
            self.set_group(self.sol, g, coef)

    def stable_dt(self, cfl: float = 0.1, lam: float = 1.0) -> float:
        pmax = max(g.p for g in self.groups)
        return cfl * self.mesh.h / ((2 * pmax + 1) * lam)


def mixed_types_euler(n: int = 12, seed: int = 0, p_set=(1, 2, 3, 4), num_flux: int = NUM_FLUX_ROE_PIKE,
                      mach: float = 0.5, perturb: float = 0.05, c_blocks: float = 0.06, w_columns: float = 0.15,
                      p_tri: float = 1.0, positivity: bool = True, curved: float = 0.0) -> MixedTypeProblem:
    """Mixed HEX/TET/WEDGE/PYR mesh of the periodic unit cube (n^3 cells), p uniform in p_set per volume (seeded),
    Euler with a smooth seeded sinusoidal state around a Mach `mach` free stream (as mixed.mixed_euler). The
    positivity limiter is on by default, as the reference applies it to every Euler stage
    (test_case_requires_positivity). curved > 0 maps the cube by SineDeform(3, curved): every volume curved."""
    mesh = MixedTypeMesh(n, seed=seed, c_blocks=c_blocks, w_columns=w_columns, p_tri=p_tri)
    rng = np.random.default_rng(seed + 17)
    p_vol = rng.choice(np.asarray(p_set, dtype=np.int32), size=mesh.n_volumes)
    prob = MixedTypeProblem(mesh, p_vol, num_flux=num_flux, positivity=positivity,
                            deform=SineDeform(3, curved) if curved else None)
    rng2 = np.random.default_rng(seed + 1)
    ph = rng2.uniform(0.0, 2.0 * math.pi, size=(5, 3))
    c0 = math.sqrt(GAMMA)
    dirn = np.array([1.0, 0.5, 0.25])
    dirn /= np.linalg.norm(dirn)

    def state(x):
        def wave(k):
            s = np.ones(len(x))
            for j in range(3):
                s = s * np.sin(2.0 * math.pi * x[:, j] + ph[k, j])
            return s
        rho = 1.0 + perturb * wave(0)
        pr = 1.0 + perturb * wave(1)
        vel = np.stack([mach * c0 * dirn[j] * (1.0 + perturb * wave(2 + j)) for j in range(3)])
        return primitive_to_conserved(3, rho, vel, pr).T

    prob.project(state)
    lam = mach * c0 * (1.0 + perturb) + c0 * math.sqrt((1.0 + perturb) / (1.0 - perturb))
    prob.dt = prob.stable_dt(lam=lam)
    prob.meta.update(n=n, seed=seed, p_set=tuple(p_set), counts=mesh.counts())
    return prob


def mixed_tri_quad_euler(n: int = 16, seed: int = 0, p_set=(1, 2, 3, 4), num_flux: int = NUM_FLUX_ROE_PIKE,
                         mach: float = 0.5, perturb: float = 0.3, p_tri: float = 0.5,
                         positivity: bool = True, walls: bool = False, curved: float = 0.0) -> MixedTypeProblem:
    """Mixed QUAD/TRI mesh of the periodic unit square (n^2 cells, MixedTriQuadMesh), p uniform in p_set per volume
    (seeded), Euler with a smooth seeded sinusoidal state around a Mach `mach` free stream (as mixed_types_euler),
    positivity limiter on by default. curved > 0 maps the square by SineDeform(2, curved)."""
    mesh = MixedTriQuadMesh(n, seed=seed, p_tri=p_tri, periodic=not walls)
    rng = np.random.default_rng(seed + 17)
    p_vol = rng.choice(np.asarray(p_set, dtype=np.int32), size=mesh.n_volumes)
    prob = MixedTypeProblem(mesh, p_vol, num_flux=num_flux, positivity=positivity,
                            deform=SineDeform(2, curved) if curved else None)
    rng2 = np.random.default_rng(seed + 1)
    ph = rng2.uniform(0.0, 2.0 * math.pi, size=(4, 2))
    c0 = math.sqrt(GAMMA)
    dirn = np.array([1.0, 0.5]) / math.sqrt(1.25)

    def state(x):
        def wave(k):
            return np.sin(2.0 * math.pi * x[:, 0] + ph[k, 0]) * np.sin(2.0 * math.pi * x[:, 1] + ph[k, 1])
        rho = 1.0 + perturb * wave(0)
        pr = 1.0 + perturb * wave(1)
        vel = np.stack([mach * c0 * dirn[j] * (1.0 + perturb * wave(2 + j)) for j in range(2)])
        return primitive_to_conserved(2, rho, vel, pr).T

    prob.project(state)
    if walls:   # slip walls on the four sides of the square (BC_SLIPWALL, boundary_euler_T.c)
        prob.set_boundaries(10102)
    lam = mach * c0 * (1.0 + perturb) + c0 * math.sqrt((1.0 + perturb) / (1.0 - perturb))
    prob.dt = prob.stable_dt(lam=lam)
    prob.meta.update(n=n, seed=seed, p_set=tuple(p_set), counts=mesh.counts())
    return prob
