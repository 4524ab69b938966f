"""Per-volume and per-face geometric factors for TP meshes (caller-side set-up).

Mirrors the reference's geometry precompute (src/simulation/geometry/geometry_T.c):

* geometry is isoparametric: a Lagrange interpolant of the mapped coordinates on GLL nodes
  of order p_g = p for curved volumes and 1 for straight ones (element_operators.c:464-549,
  ``curved ? p : 1`` in geometry_T.c:740-742);
* metric terms are computed at the metric nodes vm (GLL of order p_g) and interpolated to the
  volume cubature nodes (constructor_volume_metric_terms_T, geometry_T.c:734-801); in 2D they
  are the cofactors of geometry_T.c:546-590, in 3D the conservative curl form that
  deprecated/src/setup_geom_factors.c:182-247 uses (the current reference aborts for d=3);
* the Jacobian determinant at vc comes from the Jacobian evaluated at vc directly;
* face metrics are the vm metric terms of the side-0 volume interpolated to the face cubature
  nodes; normals_fc = metrics_fc^T n_ref normalised, jacobian_det_fc = its length
  (compute_geometry_face_T geometry_T.c:274-325, compute_normals_T :412-445).

Layouts follow the reference containers: metrics_vc[v] is (n_vc, d, d) with m(n, i, j) =
J dr_j/dx_i, stored column-major per volume exactly like ``Multiarray_T`` 'C'; normals_fc is
(n_fc, d) row-major ('R').
"""
from __future__ import annotations

import numpy as np

from .element import (TPOperatorSet, gauss_lobatto, lagrange_matrix, lagrange_derivative_matrix, kron_tp,
                      tp_nodes)


def apply_nodes(op: np.ndarray, x: np.ndarray) -> np.ndarray:
    """out[v, n, ...] = sum_k op[n, k] x[v, k, ...] through batched matmul."""
    sh = x.shape
    y = np.matmul(op, x.reshape(sh[0], sh[1], -1))
    return y.reshape((sh[0], op.shape[0]) + sh[2:])


_QUAD_F_VE = ((0, 2), (1, 3), (0, 1), (2, 3))   # QUAD local faces -> vertices (element.c f_ve), v = a + 2 b


def parametric_quad_coef(vertices: np.ndarray, p: int, deform) -> np.ndarray:
    """Geometry coefficients at order p (GLL nodes) of QUAD volumes of a parametric domain from their vertices
    (n_volumes, 4, 2) in TP order: the straight bilinear positions, then parametric_quad_nodes."""
    from .element import gauss_lobatto, tp_nodes
    x_g, _ = gauss_lobatto(p + 1)
    xi = tp_nodes(x_g, 2)
    hat = [0.25 * (1.0 + sa * xi[:, 0]) * (1.0 + sb * xi[:, 1]) for sb in (-1.0, 1.0) for sa in (-1.0, 1.0)]
    straight = np.stack([sum(hat[k][None, :] * vertices[:, k, c][:, None] for k in range(4)) for c in range(2)],
                        axis=2)
    return parametric_quad_nodes(straight, x_g, deform)


def parametric_quad_nodes(X_straight: np.ndarray, x_g: np.ndarray, deform) -> np.ndarray:
    """Geometry nodes of QUAD volumes of a parametric domain, the way the reference builds them.

    compute_geom_coef_parametric_T (geometry_T.c:857-874) maps every geometry node with the domain's map, then
    correct_internal_xyz_blended_T (geometry_blended_T.c:77-96) rebuilds the volume from its straight nodes and its
    faces: constructor_xyz_blended_ce (:277-318) with use_existing_as_surf treats every local face b in order,
        xyz += blend_b * (E_b (surf_b - R_b xyz)),
    where surf_b is the mapped geometry on face b (the face's straight GLL nodes, mapped), R_b restricts volume
    nodes to the face's nodes, E_b extends a face function constantly across the volume and blend_b is the sum of
    face b's bilinear vertex functions (constructor_blend_values, :359-377). Each face sees the coordinates the
    faces before it left, so the corners end on the mapped vertices.

    X_straight: (nv, q^2, 2) straight (bilinear) positions at the GLL nodes x_g, first direction fastest.
    """
    q = len(x_g)
    rr, ss = np.tile(x_g, q), np.repeat(x_g, q)
    h = lambda t: np.stack([0.5 * (1.0 - t), 0.5 * (1.0 + t)], axis=1)
    V = np.stack([h(rr)[:, v & 1] * h(ss)[:, v >> 1] for v in range(4)], axis=1)    # vertex basis at the nodes
    X = np.array(X_straight, dtype=np.float64, copy=True)
    nv = X.shape[0]
    idx = np.arange(q)
    for b in range(4):
        # face b's nodes among the volume's: r = -1 / +1 (b = 0 / 1) or s = -1 / +1 (b = 2 / 3)
        on_face = (idx * q + (0 if b == 0 else q - 1)) if b < 2 else ((0 if b == 2 else q - 1) * q + idx)
        tang = ss if b < 2 else rr                          # the face coordinate of every volume node
        E = lagrange_matrix(x_g, tang)                      # (q^2, q)
        blend = V[:, _QUAD_F_VE[b][0]] + V[:, _QUAD_F_VE[b][1]]
        surf = deform(X_straight[:, on_face, :].reshape(-1, 2)).reshape(nv, q, 2)
        X = X + blend[None, :, None] * np.matmul(E, surf - X[:, on_face, :])
    return X


class TPGeometry:
    def __init__(self, mesh, ops: TPOperatorSet, deform=None, curved: bool | None = None, vols=None, coef=None,
                 parametric: bool = False):
        """deform: callable (m, d) physical -> (m, d) physical applied to the affine element map, or None.
        parametric (2D): build the mapped volumes as the reference does for a parametric domain (the map on the
        faces, blended into the volume: parametric_quad_nodes) instead of mapping every geometry node.
        vols: indices of the volumes to compute (all volumes and their faces when None; the volume terms only
        otherwise, as for one (type, p) group of a mixed-order mesh).
        coef: the geometry coefficients themselves, (n_volumes, n_g, d) coordinates at the GLL nodes of order p_g
        (p when curved, else 1; for straight volumes the vertices in the reference's order), instead of the affine
        box map and deform (Solver_Volume_T::geom_coef of a mesh read from a file)."""
        d = mesh.d
        self.d = d
        if curved is None:
            curved = deform is not None
        self.curved = bool(curved)
        p_g = ops.p if self.curved else 1
        self.p_g = p_g
        x_g, _ = gauss_lobatto(p_g + 1)
        xi_g = tp_nodes(x_g, d)                      # geometry == metric nodes (p_m = p_g)
        n_g = len(xi_g)
        self.x_g = x_g

        # geometry node coordinates (nv, n_g, d)
        if coef is not None:
            X = np.asarray(coef, dtype=np.float64)
            if vols is not None:
                X = X[np.asarray(vols)]
            if X.shape[1:] != (n_g, d):
                raise ValueError(f"geometry coefficients of shape {X.shape[1:]}, expected {(n_g, d)}")
            nv = len(X)
        else:
            lo = mesh.vertices_lo if vols is None else mesh.vertices_lo[np.asarray(vols)]
            nv = len(lo)
            X = lo[:, None, :] + 0.5 * (xi_g[None, :, :] + 1.0) * mesh.h[None, None, :]
            if deform is not None and parametric:
                if d != 2:
                    raise ValueError("parametric blending is built for QUAD volumes")
                X = parametric_quad_nodes(X, x_g, deform)
            elif deform is not None:
                X = deform(X.reshape(-1, d)).reshape(nv, n_g, d)
        self.X_geom = X

        L_gg = lagrange_matrix(x_g, x_g)
        D_gg = lagrange_derivative_matrix(x_g, x_g)
        L_gc = lagrange_matrix(x_g, ops.x_vc)
        D_gc = lagrange_derivative_matrix(x_g, ops.x_vc)

        def tp_op(one_d_list):
            return kron_tp(one_d_list)

        Dm = [tp_op([D_gg if k == j else L_gg for k in range(d)]) for j in range(d)]      # at vm
        Dc = [tp_op([D_gc if k == j else L_gc for k in range(d)]) for j in range(d)]      # at vc
        I_mc = tp_op([L_gc] * d)                                                          # vm -> vc

        # Jacobian at vm: Jm[v, n, i, j] = dx_i/dr_j
        Jm = np.stack([apply_nodes(Dm[j], X) for j in range(d)], axis=-1)
        Jc = np.stack([apply_nodes(Dc[j], X) for j in range(d)], axis=-1)

        m_vm = np.empty_like(Jm)
        if d == 2:
            m_vm[..., 0, 0] = Jm[..., 1, 1]
            m_vm[..., 0, 1] = -Jm[..., 1, 0]
            m_vm[..., 1, 0] = -Jm[..., 0, 1]
            m_vm[..., 1, 1] = Jm[..., 0, 0]
        else:
            for i in range(3):
                mm = (i + 1) % 3
                ll = (i + 2) % 3
                # V_j = X_l dX_m/dr_j - X_m dX_l/dr_j  (nodal products = interpolant on vm nodes)
                V = X[:, :, ll, None] * Jm[:, :, mm, :] - X[:, :, mm, None] * Jm[:, :, ll, :]
                dV = np.stack([apply_nodes(Dm[j], V) for j in range(3)], axis=-1)  # dV[..., c, j]
                curl = np.empty_like(V)
                curl[..., 0] = dV[..., 2, 1] - dV[..., 1, 2]
                curl[..., 1] = dV[..., 0, 2] - dV[..., 2, 0]
                curl[..., 2] = dV[..., 1, 0] - dV[..., 0, 1]
                m_vm[:, :, i, :] = -0.5 * curl
        self.metrics_vm = m_vm
        self.metrics_vc = apply_nodes(I_mc, m_vm)       # (nv, n_vc, d, d)
        if d == 2:
            detJ = Jc[..., 0, 0] * Jc[..., 1, 1] - Jc[..., 0, 1] * Jc[..., 1, 0]
        else:
            detJ = (Jc[..., 0, 0] * (Jc[..., 1, 1] * Jc[..., 2, 2] - Jc[..., 1, 2] * Jc[..., 2, 1])
                    - Jc[..., 0, 1] * (Jc[..., 1, 0] * Jc[..., 2, 2] - Jc[..., 1, 2] * Jc[..., 2, 0])
                    + Jc[..., 0, 2] * (Jc[..., 1, 0] * Jc[..., 2, 1] - Jc[..., 1, 1] * Jc[..., 2, 0]))
        if np.any(detJ <= 0.0):
            raise ValueError("non-positive Jacobian determinant")
        self.jacobian_det_vc = detJ                                   # (nv, n_vc)
        # xyz at vc (advection flux input, reference constructor_xyz_vc)
        self.xyz_vc = apply_nodes(I_mc, X)
        if vols is not None:
            return

        # faces: metrics of the side-0 volume at its face cubature nodes
        nf = mesh.n_faces
        n_fc = ops.n_fc
        normals = np.empty((nf, n_fc, d))
        jac_f = np.empty((nf, n_fc))
        xyz_fc = np.empty((nf, n_fc, d))
        for lf in range(2 * d):
            sel = np.nonzero(mesh.face_lf[:, 0] == lf)[0]
            if len(sel) == 0:
                continue
            nd = lf // 2
            val = np.array([-1.0 if lf % 2 == 0 else 1.0])
            one_d = [lagrange_matrix(x_g, val) if k == nd else lagrange_matrix(x_g, ops.x_fc) for k in range(d)]
            I_mf = kron_tp(one_d)                                          # (n_fc, n_g)
            vols = mesh.face_vol[sel, 0]
            m_fc = apply_nodes(I_mf, m_vm[vols])
            nref = ops.normals_ref[lf]
            nun = np.einsum("vnij,j->vni", m_fc, nref)
            nrm = np.sqrt(np.sum(nun * nun, axis=-1))
            normals[sel] = nun / nrm[..., None]
            jac_f[sel] = nrm
            xyz_fc[sel] = apply_nodes(I_mf, X[vols])
        self.normals_fc = normals
        self.jacobian_det_fc = jac_f
        self.xyz_fc = xyz_fc


def sinusoidal_deform_2d(amplitude: float, period: float):
    """x,y += A sin(2 pi x / period) sin(2 pi y / period)  (same displacement on both coordinates)."""
    k = 2.0 * np.pi / period

    def f(x):
        dlt = amplitude * np.sin(k * x[:, 0]) * np.sin(k * x[:, 1])
        return x + dlt[:, None]
    return f


def sinusoidal_deform_3d(amplitude: float, period: float, phases=(1.0, 1.0, 1.0)):
    """x_i += A_i sin(2 pi x/L) sin(2 pi y/L) sin(2 pi z/L), A_i = amplitude * phases[i]."""
    k = 2.0 * np.pi / period
    ph = np.asarray(phases, dtype=np.float64)

    def f(x):
        s = np.sin(k * x[:, 0]) * np.sin(k * x[:, 1]) * np.sin(k * x[:, 2])
        return x + amplitude * s[:, None] * ph[None, :]
    return f
