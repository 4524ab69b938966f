"""gmsh meshes: the reader and connectivity of libdgpu (include/dgpu_mesh.h) from Python, and a writer of the
reference's gmsh 2.2 dialect for structured QUAD/HEX boxes.

``GmshMesh(path, d)`` reads a file through ``dgpu_gmsh_read`` (the reference's constructor_Mesh: mesh_reader_gmsh,
constructor_Mesh_Connectivity, constructor_Mesh_Vertices, then constructor_Faces' face list) and holds its results
as numpy arrays in the reference's containers: Mesh_Data (``nodes``, ``elem_types``, ``elem_tags``, ``node_nums``,
``periodic_corr``, ``elem_per_dim``), Mesh_Connectivity (``v_to_v``, ``v_to_lf``, ``v_to_lf_wp``, per volume),
Mesh_Vertices (``ve_curved``, ``ve_boundary``, ``ve_bc``) and the face list (``face_vol``, ``face_lf``, ``face_bc``,
``face_wp``, ``face_match``, ``face_ord``).
"""
from __future__ import annotations

import ctypes

import math

import numpy as np

from .. import _lib

LINE, TRI, QUAD, TET, HEX, WEDGE, PYR, POINT = 1, 2, 3, 4, 5, 6, 7, 15


def _ip(a):
    return a.ctypes.data_as(_lib.c_int_p)


def _dp(a):
    return a.ctypes.data_as(_lib.c_double_p)


class GmshError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"dgpu status {status}: {message}")
        self.status = status


def _split(ptr, flat):
    return [flat[ptr[i]:ptr[i + 1]].copy() for i in range(len(ptr) - 1)]


class GmshMesh:
    def __init__(self, path: str, d: int):
        lib = _lib.load()
        h = ctypes.c_void_p()
        st = lib.dgpu_gmsh_read(str(path).encode(), d, ctypes.byref(h))
        if st != 0:
            raise GmshError(st, lib.dgpu_gmsh_last_error().decode())
        try:
            sz = _lib.GmshSizes()
            lib.dgpu_gmsh_get_sizes(h, ctypes.byref(sz))
            self.d = d
            self.nodes = np.empty((sz.n_nodes, d))
            self.elem_types = np.empty(sz.n_elements, np.int32)
            self.elem_tags = np.empty((sz.n_elements, 2), np.int32)
            node_ptr = np.empty(sz.n_elements + 1, np.int32)
            node_nums = np.empty(sz.n_node_nums, np.int32)
            self.periodic_corr = np.empty((sz.n_periodic, 2), np.int32)
            self.elem_per_dim = np.empty(4, np.int32)
            lib.dgpu_gmsh_data(h, _dp(self.nodes), _ip(self.elem_types), _ip(self.elem_tags), _ip(node_ptr),
                               _ip(node_nums), _ip(self.periodic_corr), _ip(self.elem_per_dim))
            self.node_nums = _split(node_ptr, node_nums)
            lf_ptr = np.empty(sz.n_volumes + 1, np.int32)
            vv, vl, vw = (np.empty(sz.n_volume_faces, np.int32) for _ in range(3))
            lib.dgpu_gmsh_connectivity(h, _ip(lf_ptr), _ip(vv), _ip(vl), _ip(vw))
            self.v_to_v, self.v_to_lf = _split(lf_ptr, vv), _split(lf_ptr, vl)
            self.v_to_lf_wp = _split(lf_ptr, vw) if sz.has_periodic else None
            self.ve_curved = np.empty(sz.n_nodes, np.int32)
            self.ve_boundary = np.empty(sz.n_nodes, np.int32)
            bc_ptr = np.empty(sz.n_nodes + 1, np.int32)
            ve_bc = np.empty(max(sz.n_ve_bc, 1), np.int32)
            lib.dgpu_gmsh_vertices(h, _ip(self.ve_curved), _ip(self.ve_boundary), _ip(bc_ptr), _ip(ve_bc))
            self.ve_bc = _split(bc_ptr, ve_bc)
            nf = sz.n_faces
            self.face_vol = np.empty((nf, 2), np.int32)
            self.face_lf = np.empty((nf, 2), np.int32)
            self.face_bc = np.empty(nf, np.int32)
            self.face_wp = np.empty(nf, np.int32)
            self.face_match = np.empty((nf, 4), np.int32)
            self.face_ord = np.empty((nf, 2), np.int32)
            lib.dgpu_gmsh_faces(h, _ip(self.face_vol), _ip(self.face_lf), _ip(self.face_bc), _ip(self.face_wp),
                                _ip(self.face_match), _ip(self.face_ord))
        finally:
            lib.dgpu_gmsh_destroy(h)
        self.n_volumes = sz.n_volumes
        self.n_faces = sz.n_faces
        self.ind_v = int(np.sum(self.elem_per_dim[:d]))

    def volume_types(self):
        return self.elem_types[self.ind_v:]

    def volume_vertices(self) -> np.ndarray:
        """(n_volumes, n_ve, d) vertex coordinates in the reference's vertex order (one element type only)."""
        return np.stack([self.nodes[self.node_nums[self.ind_v + v]] for v in range(self.n_volumes)])


# ---- writer: structured boxes in the reference's gmsh 2.2 dialect ---------------------------------------------------
_GMSH_FROM_TP = {2: [0, 1, 3, 2], 3: [0, 1, 3, 2, 4, 5, 7, 6]}   # the reordering is its own inverse


def _rotations(d):
    """The orientation-preserving signed permutations of R^d (4 in 2D, 24 in 3D)."""
    import itertools
    out = []
    for perm in itertools.permutations(range(d)):
        for signs in itertools.product((1, -1), repeat=d):
            R = np.zeros((d, d), dtype=int)
            for i, j in enumerate(perm):
                R[i, j] = signs[i]
            if round(np.linalg.det(R)) == 1:
                out.append(R)
    return out


def write_box_msh(path, d: int, n, lo=0.0, hi=1.0, periodic=True, codes=None, rotate_seed=None,
                  perturb: float = 0.0, perturb_seed: int = 0):
    """Write an n^d QUAD/HEX box [lo, hi]^d as a gmsh 2.2 file the way the reference's meshes come: boundary
    elements (dimension d-1) first, physical tag = BC code, entity tag, then the volumes (physical tag 9401).
    periodic: per direction (or one bool); periodic directions get the codes 10051/10052 (x), 10053/10054 (y),
    10055/10056 (z) and a $Periodic section; codes: {(dim, side): code} for the other sides.
    rotate_seed: give every volume a random orientation-preserving local frame (its vertex list rotated), so that
    neighbours see their common face in different orientations. perturb: move the interior vertices by up to this
    fraction of the spacing (seeded), which leaves straight but non-affine volumes."""
    n = [int(v) for v in (n if np.ndim(n) else [n] * d)]
    per = list(periodic) if np.ndim(periodic) else [bool(periodic)] * d
    lo = np.broadcast_to(np.asarray(lo, dtype=np.float64), (d,))
    hi = np.broadcast_to(np.asarray(hi, dtype=np.float64), (d,))
    h = (hi - lo) / np.array(n)
    npts = [v + 1 for v in n]
    grid = np.stack(np.meshgrid(*[lo[k] + h[k] * np.arange(npts[k]) for k in range(d)], indexing="ij"), axis=-1)
    grid = np.transpose(grid, tuple(range(d))[::-1] + (d,)).reshape(-1, d)   # node = i + (n+1) j (+ (n+1)^2 k)
    idx = np.stack(np.meshgrid(*[np.arange(v) for v in npts], indexing="ij"), axis=-1)
    idx = np.transpose(idx, tuple(range(d))[::-1] + (d,)).reshape(-1, d)
    if perturb > 0.0:
        rng = np.random.default_rng(perturb_seed)
        inner = np.all((idx > 0) & (idx < np.array(n)), axis=1)
        grid[inner] += perturb * h * rng.uniform(-1.0, 1.0, size=(int(inner.sum()), d))

    def node(ijk):
        return int(sum(int(ijk[k]) * int(np.prod(npts[:k])) for k in range(d)))

    corners = np.array([[(v >> k) & 1 for k in range(d)] for v in range(2 ** d)])   # TP vertex order
    rots = _rotations(d)
    rng = np.random.default_rng(rotate_seed) if rotate_seed is not None else None
    lines = []

    def elem(t, tags, verts):
        lines.append((t, tags, verts))

    side_codes = {}
    for k in range(d):
        for s in range(2):
            side_codes[(k, s)] = (10051 + 2 * k + s) if per[k] else codes[(k, s)]
    # boundary elements: the faces of the box, side by side
    for k in range(d):
        others = [j for j in range(d) if j != k]
        for s in range(2):
            for cell in np.ndindex(*[n[j] for j in others]):
                verts = []
                for c in corners[:2 ** (d - 1)]:
                    ijk = np.zeros(d, dtype=int)
                    ijk[k] = s * n[k]
                    for a, j in enumerate(others):
                        ijk[j] = cell[a] + c[a]
                    verts.append(node(ijk))
                t = LINE if d == 2 else QUAD
                if t == QUAD:
                    verts = [verts[i] for i in _GMSH_FROM_TP[2]]
                elem(t, (side_codes[(k, s)], 1000 + 2 * k + s), verts)
    # volumes
    for cell in np.ndindex(*n[::-1]):
        ijk0 = np.array(cell[::-1])
        R = rots[int(rng.integers(len(rots)))] if rng is not None else np.eye(d, dtype=int)
        ref = []
        for c in corners:
            rc = R @ (2 * c - 1)                 # local vertex c of the rotated frame -> physical corner
            ref.append(node(ijk0 + (rc + 1) // 2))
        elem(QUAD if d == 2 else HEX, (9401, 4001), [ref[i] for i in _GMSH_FROM_TP[d]])
    with open(path, "w") as fh:
        fh.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(grid))
        for i, x in enumerate(grid):
            fh.write("%d %s\n" % (i + 1, " ".join("%.17g" % v for v in list(x) + [0.0] * (3 - d))))
        fh.write("$EndNodes\n$Elements\n%d\n" % len(lines))
        for i, (t, tags, verts) in enumerate(lines):
            fh.write("%d %d 2 %d %d %s\n" % (i + 1, t, tags[0], tags[1], " ".join(str(v + 1) for v in verts)))
        fh.write("$EndElements\n")
        pk = [k for k in range(d) if per[k]]
        if pk:
            fh.write("$Periodic\n%d\n" % len(pk))
            for k in pk:
                fh.write("%d %d %d\n0\n" % (d - 1, 1000 + 2 * k + 1, 1000 + 2 * k))
            fh.write("$EndPeriodic\n")


def write_annulus_msh(path, n_r: int, n_t: int, r_i: float = 0.5, r_o: float = 1.0, inner: int = 20113,
                      outer: int = 20111, rotate_seed=None):
    """Write the QUAD annulus r_i <= r <= r_o (n_r volumes across, n_t around, vertices on the circles) as a gmsh 2.2
    file the way the reference's n-cylinder_hollow meshes come: the boundary lines on r_i and r_o carry the codes
    inner and outer (BC_CURVED_START + code: curved, e.g. 20113 for the rotating wall), then the volumes. The mesh is
    conforming round the circle (no periodic section). rotate_seed: random local frames, as in write_box_msh."""
    def node(i, j):
        return i + (n_r + 1) * (j % n_t)

    pts = []
    for j in range(n_t):
        th = 2.0 * math.pi * j / n_t
        for i in range(n_r + 1):
            r = r_i + (r_o - r_i) * i / n_r
            pts.append((r * math.cos(th), r * math.sin(th)))
    rots = _rotations(2)
    rng = np.random.default_rng(rotate_seed) if rotate_seed is not None else None
    corners = np.array([[v & 1, (v >> 1) & 1] for v in range(4)])
    lines = []
    for j in range(n_t):
        lines.append((LINE, (inner, 1001), [node(0, j), node(0, j + 1)]))
    for j in range(n_t):
        lines.append((LINE, (outer, 1002), [node(n_r, j), node(n_r, j + 1)]))
    for j in range(n_t):
        for i in range(n_r):
            R = rots[int(rng.integers(len(rots)))] if rng is not None else np.eye(2, dtype=int)
            ref = []
            for c in corners:
                rc = (R @ (2 * c - 1) + 1) // 2
                ref.append(node(i + int(rc[0]), j + int(rc[1])))
            lines.append((QUAD, (9401, 4001), [ref[k] for k in _GMSH_FROM_TP[2]]))
    with open(path, "w") as fh:
        fh.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(pts))
        for k, (x, y) in enumerate(pts):
            fh.write("%d %.17g %.17g 0\n" % (k + 1, x, y))
        fh.write("$EndNodes\n$Elements\n%d\n" % len(lines))
        for k, (t, tags, verts) in enumerate(lines):
            fh.write("%d %d 2 %d %d %s\n" % (k + 1, t, tags[0], tags[1], " ".join(str(v + 1) for v in verts)))
        fh.write("$EndElements\n")


def write_square_annulus_msh(path, n_t: int, n_r: int, r_i: float = 0.5, r_o: float = 1.0, inner: int = 20113,
                             outer: int = 20111):
    """Write the square annulus r_i <= max(|x|, |y|) <= r_o as a QUAD gmsh 2.2 file, the parametric domain of the
    reference's n-cylinder_hollow/2d.geo (mesh_domain PARAMETRIC: the squares of half-sides r_i and r_o, four
    transfinite blocks split along the diagonals) that its cylinder map takes to the circular annulus. n_t volumes
    along each side of a block, n_r across; the boundary lines of the inner and outer squares carry the codes inner
    and outer (as the .geo's Physical Lines: 2 BC_STEP_SC + BC_NOSLIP_ALL_ROTATING inside, + BC_NOSLIP_ADIABATIC or
    BC_NOSLIP_DIABATIC outside), then the volumes, all with the same local frame (r radial, s counter-clockwise)."""
    n_a = 4 * n_t

    def node(i, j):
        return i + (n_r + 1) * (j % n_a)

    pts = []
    for j in range(n_a):
        side, a = divmod(j, n_t)
        a = a / n_t
        for i in range(n_r + 1):
            r = r_i + (r_o - r_i) * i / n_r
            pts.append(((-r + 2.0 * r * a, -r), (r, -r + 2.0 * r * a), (r - 2.0 * r * a, r),
                        (-r, r - 2.0 * r * a))[side])
    elems = []
    for j in range(n_a):
        elems.append((LINE, (inner, 1001), [node(0, j), node(0, j + 1)]))
    for j in range(n_a):
        elems.append((LINE, (outer, 1005), [node(n_r, j), node(n_r, j + 1)]))
    for j in range(n_a):
        for i in range(n_r):   # gmsh's counter-clockwise order
            elems.append((QUAD, (9401, 4001), [node(i, j), node(i + 1, j), node(i + 1, j + 1), node(i, j + 1)]))
    with open(path, "w") as fh:
        fh.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(pts))
        for k, (x, y) in enumerate(pts):
            fh.write("%d %.17g %.17g 0\n" % (k + 1, x, y))
        fh.write("$EndNodes\n$Elements\n%d\n" % len(elems))
        for k, (t, tags, verts) in enumerate(elems):
            fh.write("%d %d 2 %d %d %s\n" % (k + 1, t, tags[0], tags[1], " ".join(str(v + 1) for v in verts)))
        fh.write("$EndElements\n")


def write_quarter_square_annulus_msh(path, n_t: int, n_r: int, r_i: float = 1.0, r_o: float = 1.384,
                                     radial: int = 10101, inner: int = 20102, outer: int = 30102):
    """Write the quarter square annulus x, y >= 0, r_i <= max(x, y) <= r_o as a QUAD gmsh 2.2 file, the parametric
    domain of the reference's n-cylinder_hollow_section/2d.geo (mesh_domain PARAMETRIC: two transfinite blocks split
    along the diagonal from (r_i, r_i) to (r_o, r_o)) that its cylinder map takes to the quarter annulus. n_t volumes
    along each side of a block, n_r across; the boundary lines carry the .geo's Euler codes: radial (the lines on
    y = 0 and x = 0, BC_STEP_SC + BC_RIEMANN), inner (2 BC_STEP_SC + BC_SLIPWALL) and outer (3 BC_STEP_SC +
    BC_SLIPWALL). Then the volumes, all with the same local frame (r radial, s counter-clockwise)."""
    n_a = 2 * n_t

    def node(i, j):
        return i + (n_r + 1) * j

    pts = []
    for j in range(n_a + 1):
        for i in range(n_r + 1):
            r = r_i + (r_o - r_i) * i / n_r
            pts.append((r, r * j / n_t) if j <= n_t else (r - r * (j - n_t) / n_t, r))
    elems = []
    for i in range(n_r):
        elems.append((LINE, (radial, 1001), [node(i, 0), node(i + 1, 0)]))
    for i in range(n_r):
        elems.append((LINE, (radial, 1002), [node(i, n_a), node(i + 1, n_a)]))
    for j in range(n_a):
        elems.append((LINE, (inner, 1003), [node(0, j), node(0, j + 1)]))
    for j in range(n_a):
        elems.append((LINE, (outer, 1005), [node(n_r, j), node(n_r, j + 1)]))
    for j in range(n_a):
        for i in range(n_r):   # gmsh's counter-clockwise order
            elems.append((QUAD, (9401, 4001), [node(i, j), node(i + 1, j), node(i + 1, j + 1), node(i, j + 1)]))
    with open(path, "w") as fh:
        fh.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(pts))
        for k, (x, y) in enumerate(pts):
            fh.write("%d %.17g %.17g 0\n" % (k + 1, x, y))
        fh.write("$EndNodes\n$Elements\n%d\n" % len(elems))
        for k, (t, tags, verts) in enumerate(elems):
            fh.write("%d %d 2 %d %d %s\n" % (k + 1, t, tags[0], tags[1], " ".join(str(v + 1) for v in verts)))
        fh.write("$EndElements\n")


# ---- a TP problem on a mesh read from a file ------------------------------------------------------------------------
def tp_face_permutation(match, q: int, d: int) -> np.ndarray:
    """The right-trace gather permutation nc (sR[i] = sR_own[nc[i]]) of a TP face's q^(d-1) GL nodes from the
    vertex correspondence `match` (side 0's face vertex i is side 1's vertex match[i], both in TP face-vertex order,
    vertex bits = face coordinates). The correspondence fixes the map between the two sides' face coordinates, a
    symmetry of the reference segment or square; the symmetric GL nodes follow it (x_{q-1-a} = -x_a)."""
    a = np.arange(q)
    if d == 2:
        return (a[::-1] if match[0] == 1 else a).astype(np.int32)

    def c(j):
        return np.array([2 * (j & 1) - 1, 2 * ((j >> 1) & 1) - 1])
    A0 = (c(match[1]) - c(match[0])) // 2       # image of side 0's first face axis in side 1's coordinates
    A1 = (c(match[2]) - c(match[0])) // 2
    nc = np.empty(q * q, dtype=np.int32)
    for b in range(q):
        for aa in range(q):
            idx = []
            for k in range(2):
                if A0[k] != 0:
                    idx.append(aa if A0[k] > 0 else q - 1 - aa)
                else:
                    idx.append(b if A1[k] > 0 else q - 1 - b)
            nc[aa + q * b] = idx[0] + q * idx[1]
    return nc


class GmshTPMesh:
    """The face list and geometry coefficients of an all-QUAD (d = 2) or all-HEX (d = 3) mesh read from a file, with
    the attributes the problem builders use (face_vol, face_lf, h, ...)."""

    def __init__(self, gm: GmshMesh):
        d = gm.d
        t = QUAD if d == 2 else HEX
        if not np.all(gm.volume_types() == t):
            raise ValueError("the uniform TP path takes all-QUAD (d = 2) or all-HEX (d = 3) meshes")
        self.gmsh = gm
        self.d = d
        self.e_type = t
        self.n_volumes = gm.n_volumes
        self.n_faces = gm.n_faces
        self.face_vol = gm.face_vol.copy()
        self.face_lf = gm.face_lf.copy()
        self.face_bc = gm.face_bc.copy()
        self.vertices = gm.volume_vertices()                     # (n_volumes, 2^d, d), TP order
        edges = [np.linalg.norm(self.vertices[:, 1 << k] - self.vertices[:, 0], axis=1) for k in range(d)]
        self.h = np.array([float(np.min(e)) for e in edges])

    def nc_fc(self, q: int) -> np.ndarray:
        nf = q ** (self.d - 1)
        nc = np.tile(np.arange(nf, dtype=np.int32), (self.n_faces, 1))
        for f in np.nonzero(self.face_vol[:, 1] >= 0)[0]:
            nc[f] = tp_face_permutation(self.gmsh.face_match[f], q, self.d)
        return nc


BC_CURVED_START = 20000   # definitions_bc.h:34: codes above it mark curved boundary faces


def curved_faces(mesh) -> np.ndarray:
    """(n_volumes, 2d): 1 where a volume's local face is a curved boundary face (face_bc > BC_CURVED_START,
    is_face_bc_curved), the faces a blended domain moves onto its surface."""
    fc = np.zeros((mesh.n_volumes, 2 * mesh.d), dtype=np.int32)
    for f in np.nonzero((mesh.face_vol[:, 1] < 0) & (mesh.face_bc > BC_CURVED_START))[0]:
        fc[mesh.face_vol[f, 0], mesh.face_lf[f, 0]] = 1
    return fc


def gmsh_tp_problem(path, d: int, p: int, pde: int, num_flux: int, state, b_adv=(1.0, 0.5, 0.0), exterior=None,
                    bc_data=None, cfl: float = 0.1, name: str | None = None, ns=None, blend=None, parametric=None):
    """A DGProblem on the QUAD/HEX mesh in a gmsh file: geometry coefficients = the volumes' vertices (p_g = 1),
    state(xyz (m, d)) -> (m, n_var) the conserved initial state at the solution nodes, exterior(xyz) likewise the
    exterior state of the boundary faces (their BC codes come from the file), bc_data the BC_Data scalars, ns the
    Navier-Stokes constants (pde 4). blend(xyz_ve (n_volumes, 2, 4), face_curved, p) -> (n_volumes, (p+1)^2, 2):
    the blended domain's geometry coefficients at order p for the volumes with curved faces (2D; e.g.
    solver.blend_geometry on the device). parametric(xy (m, 2)) -> (m, 2): the domain map of a parametric QUAD mesh,
    applied as the reference applies it (geometry.parametric_quad_nodes: the map on every face, blended into the
    volume) at p_g = p."""
    from .element import TPOperatorSet
    from .geometry import TPGeometry
    from .problem import DGProblem, PDE_ADVECTION, stable_dt
    gm = GmshMesh(path, d)
    mesh = GmshTPMesh(gm)
    ops = TPOperatorSet(mesh.e_type, p)
    if blend is not None:
        coef = blend(np.ascontiguousarray(np.transpose(mesh.vertices, (0, 2, 1))), curved_faces(mesh), p)
        geom = TPGeometry(mesh, ops, curved=True, coef=coef)
    elif parametric is not None:
        from .geometry import parametric_quad_coef
        if d != 2:
            raise ValueError("parametric meshes are built for QUAD volumes")
        geom = TPGeometry(mesh, ops, curved=True, coef=parametric_quad_coef(mesh.vertices, p, parametric))
    else:
        geom = TPGeometry(mesh, ops, curved=False, coef=mesh.vertices)
    n_var = 1 if pde == PDE_ADVECTION else d + 2
    prob = DGProblem(name or f"gmsh_{d}d", d, pde, num_flux, pde != PDE_ADVECTION, np.asarray(b_adv, dtype=np.float64),
                     ops, mesh, geom, sol=np.zeros((mesh.n_volumes, n_var, ops.n_vs)), dt=0.0, n_steps=100, ns=ns)
    xyz = prob.solution_node_xyz()
    U = np.asarray(state(xyz.reshape(-1, d)), dtype=np.float64).reshape(mesh.n_volumes, ops.n_vs, n_var)
    prob.sol = np.ascontiguousarray(np.transpose(U, (0, 2, 1)))
    if pde != PDE_ADVECTION:
        prob.dt = stable_dt(prob, cfl)
    else:
        prob.dt = cfl * float(np.min(mesh.h)) / ((2 * p + 1) * float(np.linalg.norm(prob.b_adv)))
    if np.any(mesh.face_vol[:, 1] < 0):
        if exterior is None:
            raise ValueError("the mesh has boundary faces: give their exterior state")
        prob.bc = np.where(mesh.face_vol[:, 1] < 0, mesh.face_bc, 0).astype(np.int32)
        ext = np.asarray(exterior(geom.xyz_fc.reshape(-1, d)), dtype=np.float64).reshape(mesh.n_faces, ops.n_fc, n_var)
        ext[mesh.face_vol[:, 1] >= 0] = 0.0
        prob.bc_state = np.ascontiguousarray(ext)
        prob.bc_data = bc_data
    return prob
