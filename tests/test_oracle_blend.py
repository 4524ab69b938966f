"""The oracle's restatement of the reference's blended geometry (oracle/blend.py: compute_geom_coef_blended_T with
TP Gordon-Hall blending and the n-cylinder radial projection) against what it must satisfy.

The reference's blended test meshes (n-cylinder_hollow, the Taylor-Couette case) are generated by gmsh at run time,
and the reference keeps no geometry fixtures for them, so these are known answers:
- the nodes of a curved face lie on its circle;
- a volume without curved faces keeps its bilinear map, and the straight faces of a curved volume keep theirs;
- the area of the blended annulus converges to pi (r_o^2 - r_i^2) as p_g grows;
- the fluid at rest on the blended Taylor-Couette mesh is steady.
"""
import math

import numpy as np
import pytest

import oracle
from oracle import blend as B
from dpgsolver_gb300.host import problem as P


@pytest.mark.parametrize("p_g", [1, 2, 3, 4])
def test_curved_faces_on_their_circles_and_straight_faces_kept(p_g):
    ve, fc = P.annulus_vertices(6, rotate=0.3)
    g = B.blend_quad(ve, fc, p_g)
    q = p_g + 1
    x = B.gll_nodes(q)
    straight = np.einsum("nv,evc->ecn", B.vertex_basis(np.tile(x, q), np.repeat(x, q)), np.transpose(ve, (0, 2, 1)))
    r = np.hypot(g[:, 0], g[:, 1]).reshape(len(ve), q, q)          # [v][j][i]
    for v in range(len(ve)):
        if fc[v, 0]:
            assert np.max(np.abs(r[v, :, 0] - 0.5)) < 1e-15
        if fc[v, 1]:
            assert np.max(np.abs(r[v, :, q - 1] - 1.0)) < 1e-15
        sv = straight[v].reshape(2, q, q)
        gv = g[v].reshape(2, q, q)
        # the faces s = -1 and s = +1 (local faces 2, 3) are straight radial lines: kept
        assert np.max(np.abs(gv[:, 0, :] - sv[:, 0, :])) < 1e-15
        assert np.max(np.abs(gv[:, q - 1, :] - sv[:, q - 1, :])) < 1e-15


def test_volume_without_curved_faces_is_bilinear():
    ve, fc = P.annulus_vertices(4)
    g = B.blend_quad(ve, np.zeros_like(fc), 3)
    x = B.gll_nodes(4)
    straight = np.einsum("nv,evc->ecn", B.vertex_basis(np.tile(x, 4), np.repeat(x, 4)), np.transpose(ve, (0, 2, 1)))
    assert np.max(np.abs(g - straight)) < 1e-15


def _area(n, p):
    from dpgsolver_gb300.host.element import TPOperatorSet
    from dpgsolver_gb300.host.geometry import TPGeometry
    from dpgsolver_gb300.host.mesh import StructuredMesh
    ve, fc = P.annulus_vertices(n)
    mesh = StructuredMesh(2, n, 0.0, 1.0, periodic=(False, True))
    ops = TPOperatorSet(mesh.e_type, p)
    geom = TPGeometry(mesh, ops, curved=True, coef=np.transpose(B.blend_quad(ve, fc, p), (0, 2, 1)))
    return float((geom.jacobian_det_vc * ops.w_vc[None, :]).sum())


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_blended_annulus_area_converges_at_h_to_the_2p(p):
    """Halving h divides the area error by at least 0.8 * 2^(2p) (measured 3.9, 15.8, 68, 270 for p = 1..4)."""
    exact = math.pi * (1.0 - 0.25)
    e8, e16 = (abs(_area(n, p) - exact) for n in (8, 16))
    assert e16 < e8 / (0.8 * 2.0 ** (2 * p))


def test_taylor_couette_at_rest_on_the_blended_mesh_is_steady():
    """The raw residual of the fluid at rest is rounding (the blended volumes next to the walls are thinner than
    the polar map's, so M^-1 amplifies it more)."""
    ve, fc = P.annulus_vertices((3, 16))
    coef = np.transpose(B.blend_quad(ve, fc, 3), (0, 2, 1))
    prob = P.ns_taylor_couette((3, 16), 3, mu=0.02, omega=0.0, geom_coef=coef)
    rest = P.constant_state(prob, [1.0, 0.0, 0.0, 1.0 / P.GM1])
    o = oracle.Oracle(prob)
    assert np.max(np.abs(o.compute_rhs_raw(rest))) < 1e-14
    assert o.compute_rhs(rest)[1] < 1e-11
