"""The reference's blended geometry of curved QUAD volumes, restated with dense operators in numpy.

Test infrastructure only: the tests and nothing else use it, as the checker of dgpu_blend_geometry.

It follows compute_geom_coef_blended_T (src/simulation/geometry/geometry_T.c:845-855). The straight volume is
taken at the geometry nodes (constructor_xyz_s_ho_T). constructor_xyz_blended_ce (geometry_blended_T.c:286-315)
then treats every curved boundary face b in local-face order:
    surf_diff = xyz_surface - vv0_vgc_fgc[b] xyz                (constructor_xyz_surf_diff_T :231-270)
    xyz      += blend_b * (vv0_fgc_vgc[b] surf_diff)             (constructor_xyz_diff_T :353-367)
Here blend_b is the sum of the face's vertex basis functions at the geometry nodes, the TP case of
constructor_blend_values (:337-351). xyz_surface is the radial projection of the face's straight nodes onto the
circle through the volume's first vertex on the face (constructor_xyz_surface_cylinder_radial_proj_T and
compute_radius_from_xyz_ve, geometry_surface_T.c:103-147, 179-238). Each operator is a dense matrix of Lagrange or
vertex-basis values, as in the reference's Geometry_Element.
"""
from __future__ import annotations

import numpy as np

F_VE = ((0, 2), (1, 3), (0, 1), (2, 3))   # QUAD local faces -> vertices (element.c f_ve), vertex v = a + 2 b
EPS = 1e-15                               # definitions_tol.h


def gll_nodes(q: int) -> np.ndarray:
    """Gauss-Lobatto-Legendre nodes on [-1, 1]: the end points and the roots of P'_{q-1}."""
    if q == 2:
        return np.array([-1.0, 1.0])
    inner = np.polynomial.legendre.Legendre.basis(q - 1).deriv().roots()
    return np.concatenate([[-1.0], np.sort(inner.real), [1.0]])


def lagrange(xn: np.ndarray, x: np.ndarray) -> np.ndarray:
    """L[k, a] = l_a(x[k]) for the Lagrange basis on the nodes xn."""
    L = np.ones((len(x), len(xn)))
    for a in range(len(xn)):
        for m in range(len(xn)):
            if m != a:
                L[:, a] *= (x - xn[m]) / (xn[a] - xn[m])
    return L


def vertex_basis(r: np.ndarray, s: np.ndarray) -> np.ndarray:
    """Bilinear vertex basis of the QUAD at the points (r, s): (n, 4), vertex v = a + 2 b."""
    hr = np.stack([0.5 * (1.0 - r), 0.5 * (1.0 + r)], axis=1)
    hs = np.stack([0.5 * (1.0 - s), 0.5 * (1.0 + s)], axis=1)
    return np.stack([hr[:, v & 1] * hs[:, v >> 1] for v in range(4)], axis=1)


def _face_coords(b: int, t: np.ndarray):
    one = np.ones_like(t)
    return {0: (-one, t), 1: (one, t), 2: (t, -one), 3: (t, one)}[b]


def blend_quad(xyz_ve: np.ndarray, face_curved: np.ndarray, p_g: int) -> np.ndarray:
    """xyz_ve (n_volumes, 2, 4), face_curved (n_volumes, 4) -> geom_coef (n_volumes, 2, (p_g+1)^2), GLL nodes of
    order p_g in TP order (first direction fastest)."""
    q = p_g + 1
    xg = gll_nodes(q)
    rr, ss = np.tile(xg, q), np.repeat(xg, q)              # node n = i + q j at (xg[i], xg[j])
    V_vg = vertex_basis(rr, ss)                             # vv0_vv_vg
    ops = []
    for b in range(4):
        fr, fs = _face_coords(b, xg)
        R = np.stack([np.kron(lagrange(xg, fs[k:k + 1])[0], lagrange(xg, fr[k:k + 1])[0])            # vv0_vgc_fgc
                      for k in range(q)])
        tang = ss if b < 2 else rr
        E = lagrange(xg, tang)                                                                      # vv0_fgc_vgc
        V_f = vertex_basis(fr, fs)                                                                  # vv0_vv_fgc
        blend = V_vg[:, F_VE[b][0]] + V_vg[:, F_VE[b][1]]
        ops.append((R, E, V_f, blend))
    out = np.empty((len(xyz_ve), 2, q * q))
    for v in range(len(xyz_ve)):
        ve = np.asarray(xyz_ve[v], dtype=np.float64).T      # (4, 2)
        xyz = V_vg @ ve
        for b in range(4):
            if not face_curved[v, b]:
                continue
            R, E, V_f, blend = ops[b]
            xb = V_f @ ve                                   # the face's straight nodes
            r = None
            for n in range(4):                              # find_boundary_vertex_index: first vertex on the face
                if np.min(np.max(np.abs(xb - ve[n]), axis=1)) < EPS:
                    r = float(np.sqrt(ve[n, 0] ** 2 + ve[n, 1] ** 2))
                    break
            th = np.arctan2(xb[:, 1], xb[:, 0])
            surf = np.stack([r * np.cos(th), r * np.sin(th)], axis=1)
            xyz = xyz + blend[:, None] * (E @ (surf - R @ xyz))
        out[v] = xyz.T
    return out
