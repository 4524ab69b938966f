"""Caller-side set-up: face list rule, geometry and packing invariants (CPU only)."""
import numpy as np
import pytest

from dpgsolver_gb300.host import problem as P
from dpgsolver_gb300.host.element import TPOperatorSet, QUAD, HEX
from dpgsolver_gb300.host.geometry import TPGeometry
from dpgsolver_gb300.host.mesh import StructuredMesh


@pytest.mark.parametrize("d,n", [(2, 4), (3, 3), (2, 2)])
def test_face_list_follows_reference_rule(d, n):
    """Faces are created in volume order, local-face order; the first volume met is side 0
    (computational_elements/face.c:86-160)."""
    m = StructuredMesh(d, n, 0.0, 1.0)
    assert m.n_faces == d * m.n_volumes
    seen = set()
    expect = []
    for v in range(m.n_volumes):
        for lf in range(2 * d):
            f = m.vol_faces[v, lf]
            if f not in seen:
                seen.add(f)
                expect.append(f)
                assert m.face_vol[f, 0] == v and m.face_lf[f, 0] == lf
    assert expect == list(range(m.n_faces))
    # every (volume, local face) appears exactly once
    pairs = {(int(a), int(b)) for a, b in zip(m.face_vol.ravel(), m.face_lf.ravel())}
    assert len(pairs) == 2 * m.n_faces


def test_affine_geometry_metrics_exact():
    m = StructuredMesh(2, 3, [0.0, 0.0], [3.0, 1.5])
    ops = TPOperatorSet(QUAD, 3)
    g = TPGeometry(m, ops)
    hx, hy = 0.5, 0.25  # dx/dr, dy/ds
    assert np.allclose(g.jacobian_det_vc, hx * hy)
    assert np.allclose(g.metrics_vc[..., 0, 0], hy)
    assert np.allclose(g.metrics_vc[..., 1, 1], hx)
    assert np.allclose(g.metrics_vc[..., 0, 1], 0.0) and np.allclose(g.metrics_vc[..., 1, 0], 0.0)


def test_curl_form_metrics_affine_3d():
    m = StructuredMesh(3, 2, [0.0] * 3, [2.0, 4.0, 6.0])
    ops = TPOperatorSet(HEX, 2)
    g = TPGeometry(m, ops)
    h = np.array([0.5, 1.0, 1.5])
    J = np.prod(h)
    assert np.allclose(g.jacobian_det_vc, J)
    for i in range(3):
        for j in range(3):
            expect = J / h[i] if i == j else 0.0
            assert np.allclose(g.metrics_vc[..., i, j], expect, atol=1e-13)


def test_face_normals_opposite_and_unit():
    prob = P.euler_hex_3d(3, 3)
    g = prob.geom
    assert np.allclose(np.linalg.norm(g.normals_fc, axis=-1), 1.0)
    # side-0 normals point out of the side-0 volume: along +/- the reference face normal direction
    for f in range(prob.mesh.n_faces):
        lf = prob.mesh.face_lf[f, 0]
        sgn = -1.0 if lf % 2 == 0 else 1.0
        assert np.all(sgn * g.normals_fc[f, :, lf // 2] > 0.9)


def test_problem_sizes_match_workloads():
    a = P.advection_2d()
    assert a.n_state == 2304 and a.mesh.n_faces == 512
    assert abs(a.dt - 0.1 * 0.125 / np.hypot(1.0, 0.5)) < 1e-15


def test_entropy_error_functional():
    """compute_error_euler.c's entropy error: zero for an isentropic constant state, and at the interpolation-error
    level for the projected isentropic vortex."""
    from dpgsolver_gb300.host.errors import l2_entropy_error
    prob = P.euler_vortex_2d(8, 3)
    s = P.constant_state(prob, [1.3, 0.3, -0.2, 1.3 ** 1.4 / 0.4 + 0.5 * (0.3 ** 2 + 0.2 ** 2) / 1.3])
    assert l2_entropy_error(prob, s) < 1e-14
    e0 = l2_entropy_error(prob, prob.sol)
    assert 0.0 < e0 < 1e-2
    assert l2_entropy_error(P.euler_vortex_2d(16, 3), P.euler_vortex_2d(16, 3).sol) < e0
