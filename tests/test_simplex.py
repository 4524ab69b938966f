"""Non-TP reference elements (TET, WEDGE, PYR), the mixed-type mesh and the oracle on it (CPU)."""
import math

import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import simplex as S
from dpgsolver_gb300.host.element import HEX, PYR, QUAD, TET, TRI, WEDGE, TPOperatorSet
from dpgsolver_gb300.host import mixed_types as MT

TYPES = (TET, WEDGE, PYR)
VOLUMES = {TET: 8.0 / (6.0 * math.sqrt(2.0)), WEDGE: 2.0 * math.sqrt(3.0), PYR: 4.0 * math.sqrt(2.0) / 3.0}


@pytest.mark.parametrize("alpha", [1.0, 2.0])
def test_gauss_jacobi_moments(alpha):
    from scipy.integrate import quad
    x, w = S.gauss_jacobi(5, alpha)
    for k in range(10):
        exact = quad(lambda t: (1 - t) ** alpha * t ** k, -1, 1)[0]
        assert abs(np.sum(w * x ** k) - exact) < 1e-14


@pytest.mark.parametrize("e", TYPES)
def test_volume_rules(e):
    """The reference volumes, for every order."""
    for q in (2, 3, 4, 5):
        x, w = S.volume_rule(e, q)
        assert abs(w.sum() - VOLUMES[e]) < 1e-13


@pytest.mark.parametrize("e", [TRI, TET])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_witherden_vincent_rules_are_the_references(e, p):
    """The reference's simplex cubature (Witherden-Vincent of degree 2p): the point counts of its tables, points
    inside the element, and every monomial moment up to degree 2p of the simplex, through the affine map from the
    standard simplex (the tables carry 15 significant digits)."""
    x, w = S.volume_rule(e, p + 1)
    d = 2 if e == TRI else 3
    assert len(w) == {TRI: [3, 6, 12, 16], TET: [4, 14, 24, 46]}[e][p - 1]
    assert np.all(w > 0)
    src = S._T2 if e == TRI else S._T3
    A, b = S._affine_from(src, S.TRI_VERTS if e == TRI else S.VERTS[TET])
    xs = np.linalg.solve(A, (x - b).T).T + 1.0          # standard simplex shifted to [0, 2]
    assert np.all(xs > -1e-12) and np.all(xs.sum(1) < 2.0 + 1e-12)
    import itertools
    for ex_ in itertools.product(range(2 * p + 1), repeat=d):
        if sum(ex_) > 2 * p:
            continue
        # int over {u_i >= 0, sum u <= 2} of prod u_i^a_i = 2^(sum a + d) prod a_i! / (sum a + d)!
        exact = 2.0 ** (sum(ex_) + d) * np.prod([math.factorial(a) for a in ex_]) \
            / math.factorial(sum(ex_) + d) * abs(np.linalg.det(A))
        got = np.sum(w * np.prod([xs[:, k] ** ex_[k] for k in range(d)], axis=0))
        assert abs(got - exact) < 1e-13 * max(1.0, exact), (ex_, got, exact)


@pytest.mark.parametrize("q", [2, 3, 4, 5])
def test_pyramid_rule_exact_to_degree_2p_plus_1(q):
    """The PYR keeps the conical Gauss-Jacobi rule: the volume and the moments of z^k on the reference pyramid."""
    x, w = S.volume_rule(PYR, q)
    assert len(w) == q ** 3 and abs(w.sum() - VOLUMES[PYR]) < 1e-13


@pytest.mark.parametrize("e", TYPES)
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_orthonormal_basis_and_gradients(e, p):
    o = S.DenseOperatorSet(e, p)
    assert o.n_vs == {TET: (p + 1) * (p + 2) * (p + 3) // 6, WEDGE: (p + 1) ** 2 * (p + 2) // 2,
                      PYR: (p + 1) * (p + 2) * (2 * p + 3) // 6}[e]
    assert np.abs(o.mass() - np.eye(o.n_vs)).max() < 1e-12
    x0 = o.x_vc[::7]
    _, G = o.basis(x0)
    h = 1e-6
    for k in range(3):
        dx = np.zeros(3)
        dx[k] = h
        fd = (o.basis(x0 + dx)[0] - o.basis(x0 - dx)[0]) / (2 * h)
        assert np.abs(fd - G[k]).max() < 1e-6 * max(1.0, np.abs(G[k]).max())


@pytest.mark.parametrize("e", TYPES)
def test_reference_normals_match_geometry(e):
    nr = S.reference_normals_3d(e)
    V = S.VERTS[e]
    cen = V.mean(0)
    for lf, fv in enumerate(S.F_VE[e]):
        P = V[fv]
        n = np.cross(P[1] - P[0], P[2] - P[0])
        n /= np.linalg.norm(n)
        if np.dot(n, P[0] - cen) < 0:
            n = -n
        assert np.abs(n - nr[lf]).max() < 1e-14


@pytest.mark.parametrize("e", TYPES)
def test_faces_congruent_to_face_reference(e):
    """Every face of the reference element has the area of its face reference element, so face-rule weights
    and J_f = |m n_ref| measure it consistently; face points lie on the face plane."""
    o = S.DenseOperatorSet(e, 2)
    nr = S.reference_normals_3d(e)
    for lf, fv in enumerate(S.F_VE[e]):
        P = S.VERTS[e][fv]
        if len(fv) == 3:
            area = 0.5 * np.linalg.norm(np.cross(P[1] - P[0], P[2] - P[0]))
            assert abs(area - math.sqrt(3.0)) < 1e-14
        else:
            area = np.linalg.norm(np.cross(P[1] - P[0], P[2] - P[0]))
            assert abs(area - 4.0) < 1e-14
        assert abs(o.w_fc(lf, 3).sum() - area) < 1e-13
        for ord_ in range(o.n_ords(lf)):
            x = o.face_points(lf, ord_, 3)
            assert np.abs((x - P[0]) @ nr[lf]).max() < 1e-14


def test_mixed_type_mesh_faces_match():
    """Both sides of every face evaluate at the same physical points (orientations), HEX sides unpermuted."""
    prob = MT.mixed_types_euler(4, seed=0)
    mesh = prob.mesh
    assert set(mesh.counts()) == {HEX, TET, WEDGE, PYR} and min(mesh.counts().values()) > 0
    for f in range(mesh.n_faces):
        pts = []
        for s in range(2):
            v = mesh.face_vol[f, s]
            ops = prob.groups[prob.vol_group[v]]
            lf, o = mesh.face_lf[f, s], mesh.face_ord[f, s]
            if getattr(ops, "dense", False):
                xr = ops.face_points(lf, o, int(prob.face_q[f]))
            else:
                assert o == 0
                from dpgsolver_gb300.host.element import gauss_legendre
                xq, _ = gauss_legendre(int(prob.face_q[f]))
                nd, side = lf // 2, lf % 2
                t = [k for k in range(3) if k != nd]
                xr = np.zeros((len(xq) ** 2, 3))
                xr[:, nd] = -1.0 if side == 0 else 1.0
                xr[:, t[0]] = np.tile(xq, len(xq))
                xr[:, t[1]] = np.repeat(xq, len(xq))
            pts.append(xr @ prob.A[v].T + prob.b[v])
        d = pts[0] - pts[1]
        d -= np.round(d)            # periodic images
        assert np.abs(d).max() < 1e-13


def test_mixed_type_fractions():
    """Default generator parameters give the target mix (HEX 50 %, TET 25 %, WEDGE 15 %, PYR 10 %) within a few %."""
    m = MT.MixedTypeMesh(24, seed=0)
    c = m.counts()
    tot = sum(c.values())
    for t, target in ((HEX, 0.5), (TET, 0.25), (WEDGE, 0.15), (PYR, 0.10)):
        assert abs(c[t] / tot - target) < 0.05


def _one_coefficients(ops):
    if getattr(ops, "dense", False):
        return np.linalg.solve(ops.mass(), ops.cv0_vs_vc().T @ ops.w_vc)
    return np.ones(ops.n_vs)


def test_mixed_type_oracle_free_stream_and_conservation():
    prob = MT.mixed_types_euler(4, seed=0)
    o = oracle.Oracle(prob)
    raw = o.compute_rhs_raw(prob.sol)
    tot = np.zeros(5)
    scale = np.zeros(5)
    for g, ops in enumerate(prob.groups):
        one = _one_coefficients(ops)
        B = prob.group_view(raw, g)
        tot += np.einsum("vka,a->k", B, one)
        scale += np.einsum("vka,a->k", np.abs(B), np.abs(one))
    assert np.all(np.abs(tot) <= 1e-13 * scale.max())
    vals = np.array([1.0, 0.3, -0.2, 0.1, 2.5])
    prob.project(lambda x: np.tile(vals, (len(x), 1)))
    _, mx = o.compute_rhs(prob.sol)
    assert mx < 1e-11


def test_mixed_type_complex_step():
    """Complex step = central differences on the mixed-type mesh. The additive perturbation (1e-2) keeps the two
    traces of every face node apart, away from the kinks of the numerical fluxes (max of the two sides' wave
    speeds, Roe's entropy fix), where the two linearisations legitimately differ."""
    prob = MT.mixed_types_euler(4, seed=1)
    o = oracle.Oracle(prob)
    rng = np.random.default_rng(2)
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    dirn = rng.standard_normal(prob.sol.shape)
    _, ri = o.compute_rhs_cmplx(base, 1e-30 * dirn)
    eps = 1e-6
    fd = (o.compute_rhs(base + eps * dirn)[0] - o.compute_rhs(base - eps * dirn)[0]) / (2 * eps)
    assert np.max(np.abs(ri / 1e-30 - fd)) <= 1e-6 * np.max(np.abs(fd))


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_wedge_operators_are_kronecker_products(p):
    """The WEDGE basis is the product of an orthonormal TRI basis and normalised Legendre polynomials, so its volume
    operators are Kronecker products of the TRI and LINE factors (what the sum-factorised kernel applies)."""
    o = S.DenseOperatorSet(WEDGE, p)
    t0, t1, l0, l1 = o.prism_factors()
    scale = max(np.abs(o.cv1_vs_vc(k)).max() for k in range(3))
    assert np.abs(np.kron(l0, t0) - o.cv0_vs_vc()).max() <= 1e-13 * scale
    assert np.abs(np.kron(l0, t1[0]) - o.cv1_vs_vc(0)).max() <= 1e-13 * scale
    assert np.abs(np.kron(l0, t1[1]) - o.cv1_vs_vc(1)).max() <= 1e-13 * scale
    assert np.abs(np.kron(l1, t0) - o.cv1_vs_vc(2)).max() <= 1e-13 * scale


# ---- 2D: TRI volumes and the mixed QUAD/TRI mesh ---------------------------------------------------------------------
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_tri_basis_rule_and_faces(p):
    """Orthonormal P_p on the reference TRI (element.c vertices), finite-difference gradients, face nodes on the
    face lines, face weights summing to the edge length 2, outward normals."""
    from dpgsolver_gb300.host.element import TRI
    o = S.DenseOperatorSet(TRI, p)
    assert o.n_vs == (p + 1) * (p + 2) // 2 and o.d == 2
    assert np.abs(o.mass() - np.eye(o.n_vs)).max() < 1e-12
    x0 = o.x_vc[::3]
    _, G = o.basis(x0)
    for k in range(2):
        dx = np.zeros(2)
        dx[k] = 1e-6
        fd = (o.basis(x0 + dx)[0] - o.basis(x0 - dx)[0]) / 2e-6
        assert np.abs(fd - G[k]).max() < 1e-6 * max(1.0, np.abs(G[k]).max())
    V = S.VERTS[TRI]
    for lf, fv in enumerate(S.F_VE[TRI]):
        P = V[fv]
        assert abs(o.w_fc(lf, 3).sum() - np.linalg.norm(P[1] - P[0])) < 1e-14
        t = (P[1] - P[0]) / np.linalg.norm(P[1] - P[0])
        n = np.array([t[1], -t[0]])
        if np.dot(n, P[0] - V.mean(0)) < 0:
            n = -n                                                 # outward
        assert np.abs(n - o.normals_ref[lf]).max() < 1e-14
        for ord_ in range(o.n_ords(lf)):
            assert np.abs((o.face_points(lf, ord_, 3) - P[0]) @ n).max() < 1e-14


def test_tri_quad_mesh_faces_match():
    """Both sides of every edge evaluate at the same physical points (LINE orientations), QUAD sides unpermuted."""
    from dpgsolver_gb300.host.element import QUAD, TRI, gauss_legendre
    prob = MT.mixed_tri_quad_euler(5, seed=2)
    mesh = prob.mesh
    assert mesh.counts()[TRI] > 0 and mesh.counts()[QUAD] > 0
    assert set(mesh.face_ord.ravel().tolist()) == {0, 1}
    for f in range(mesh.n_faces):
        pts = []
        for s in range(2):
            v = mesh.face_vol[f, s]
            ops = prob.groups[prob.vol_group[v]]
            lf, o = mesh.face_lf[f, s], mesh.face_ord[f, s]
            if getattr(ops, "dense", False):
                xr = ops.face_points(lf, o, int(prob.face_q[f]))
            else:
                assert o == 0
                xq, _ = gauss_legendre(int(prob.face_q[f]))
                nd, side = lf // 2, lf % 2
                xr = np.zeros((len(xq), 2))
                xr[:, nd] = -1.0 if side == 0 else 1.0
                xr[:, 1 - nd] = xq
            pts.append(xr @ prob.A[v].T + prob.b[v])
        dd = pts[0] - pts[1]
        dd -= np.round(dd)          # periodic images
        assert np.abs(dd).max() < 1e-13


def test_tri_quad_oracle_free_stream_conservation_and_complex_step():
    prob = MT.mixed_tri_quad_euler(4, seed=0)
    o = oracle.Oracle(prob)
    raw = o.compute_rhs_raw(prob.sol)
    tot, scale = np.zeros(4), np.zeros(4)
    for g, ops in enumerate(prob.groups):
        one = _one_coefficients(ops)
        B = prob.group_view(raw, g)
        tot += np.einsum("vka,a->k", B, one)
        scale += np.einsum("vka,a->k", np.abs(B), np.abs(one))
    assert np.all(np.abs(tot) <= 1e-13 * scale.max())
    rng = np.random.default_rng(3)
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    dirn = rng.standard_normal(prob.sol.shape)
    _, ri = o.compute_rhs_cmplx(base, 1e-30 * dirn)
    fd = (o.compute_rhs(base + 1e-6 * dirn)[0] - o.compute_rhs(base - 1e-6 * dirn)[0]) / 2e-6
    assert np.max(np.abs(ri / 1e-30 - fd)) <= 1e-6 * np.max(np.abs(fd))
    vals = np.array([1.0, 0.3, -0.2, 2.5])
    prob.project(lambda x: np.tile(vals, (len(x), 1)))
    assert o.compute_rhs(prob.sol)[1] < 1e-11


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_bezier_maps(p):
    """The reference's Bezier bases (bases.c:570-760) span each solution space: partition of unity, non-negative,
    the constant function has equal Bezier coefficients, and ccBS0 ccSB0 = I."""
    from dpgsolver_gb300.host.element import TRI
    for e in (TRI, TET, WEDGE, PYR):
        o = S.DenseOperatorSet(e, p)
        B = S.bezier_basis(e, p, o.x_vc)
        assert np.abs(B.sum(axis=1) - 1.0).max() < 1e-14 and B.min() >= 0.0
        sb, bs = o.ccSB0_vs_vs(), o.ccBS0_vs_vs()
        assert np.abs(bs @ sb - np.eye(o.n_vs)).max() < 1e-11
        b1 = sb @ _one_coefficients(o)
        assert np.abs(b1 - 1.0).max() < 1e-12


@pytest.mark.parametrize("make", [lambda: MT.mixed_types_euler(4, seed=1, curved=0.03),
                                  lambda: MT.mixed_tri_quad_euler(4, seed=2, curved=0.03)])
def test_curved_mixed_geometry_is_conforming(make):
    """With the SineDeform map, every face's canonical nodes seen from its two sides land on the same physical points
    (up to periodic images), and side 1's area-weighted normal there is the negative of side 0's, so the faces of the
    curved mesh close; J varies over the volumes' nodes (the dense groups are curved)."""
    from dpgsolver_gb300.host.element import TPOperatorSet, gauss_legendre
    prob = make()
    mesh, d = prob.mesh, prob.d
    nw = prob.normals_fc * prob.jacobian_det_fc[:, None]
    for f in range(mesh.n_faces):
        pts, nrm = [], []
        for s in range(2):
            v = int(mesh.face_vol[f, s])
            ops = prob.groups[prob.vol_group[v]]
            lf, o = int(mesh.face_lf[f, s]), int(mesh.face_ord[f, s])
            if getattr(ops, "dense", False):
                xr = ops.face_points(lf, o, int(prob.face_q[f]))
                nref = ops.normals_ref[lf]
            else:
                xr = MT._tp_face_points(d, lf, int(prob.face_q[f]))
                nref = TPOperatorSet(ops.e_type, 1).normals_ref[lf]
            pts.append(prob._map(np.array([v]), xr)[0])
            m, _ = prob._map_metrics(np.array([v]), xr)
            nrm.append(np.einsum("nij,j->ni", m[0], nref))
        dd = pts[0] - pts[1]
        dd -= np.round(dd)          # periodic images
        assert np.abs(dd).max() < 1e-13
        assert np.abs(nrm[0] + nrm[1]).max() < 1e-12
        assert np.abs(nrm[0] - nw[prob.face_off[f]:prob.face_off[f + 1]]).max() < 1e-13
    dense = [g for g, o in enumerate(prob.groups) if getattr(o, "dense", False)]
    assert dense and all(np.ptp(prob.J_vc[g], axis=1).min() > 0.0 for g in dense)
