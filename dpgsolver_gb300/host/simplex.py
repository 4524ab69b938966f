"""Reference-element data for the non-tensor-product 3D volumes: TET, WEDGE and PYR (caller-side set-up).

The residual kernels for these types apply dense per-element operators that the caller passes through the C
ABI, as the reference does with its op_std operators (operator_T.c:96-156). This module builds them.

Mirrored from the reference:

* Element type codes, reference-element vertices and local face numbering: the regular reference simplices and
  pyramid of element/nodes.c:474-540 (TRI vertices (-1,-1/sqrt3), (1,-1/sqrt3), (0,2/sqrt3); TET adds
  (0,0,3/sqrt6) over the plane z = -1/sqrt6; PYR: base [-1,1]^2 at z = -sqrt2/5, apex (0,0,4 sqrt2/5); WEDGE =
  TRI x [-1,1]) and the face-vertex lists f_ve of element/element.c:486-531. Every face of these reference
  elements is congruent to the face reference element (a regular triangle of side 2 or the square [-1,1]^2), so
  face cubature weights and face Jacobians are measured the same way on every type.
* Reference normals: the angle form of element/element.c:708-780.
* Default cubature degree 2p (simulation.c:494-500); the face of two volumes of orders p_L, p_R is integrated
  at p_f = max(p_L, p_R) (face_solver.c:123-132).

Choices of this set-up (the C ABI accepts any basis and cubature the caller supplies):

* Solution basis: orthonormal modal bases on the reference element (the reference uses Lagrange bases on its
  AO / GLL node sets; a change of basis does not change the discrete solution, only its coordinates). TET:
  P_p; WEDGE: P_p(TRI) x P_p(LINE); PYR: the rational pyramid space of dimension (p+1)(p+2)(2p+3)/6 spanned in
  collapsed coordinates by P_i(a) P_j(b) ((1-c)/2)^max(i,j) P_k^(2max(i,j)+2,0)(c) (Bergot-Cohen-Durufle).
* Cubature: the reference's (nodes_operators.c:313-350, 474-516, 589-609): Witherden-Vincent rules of degree 2p on
  TRI and TET volumes and on the triangular faces of 3D volumes (3/6/12/16 TRI and 4/14/24/46 TET points for
  p = 1..4, read from the reference's tables into wv_rules.npz by make_wv_rules.py), that TRI rule times GL with
  p+1 points on the WEDGE (the reference builds its operators from the TRI and LINE factors), GL with p_f+1 points
  per direction on LINE and QUAD faces. The PYR keeps a conical Gauss-Jacobi rule of (p+1)^3 points: the
  reference's own PYR choice (GJW) has no case in compute_cub_c_type, so the reference cannot build PYR operators.
  Set-up integrations that must be exact beyond degree 2p (orthonormalisation, the Bezier maps) use conical rules.
* Each face's nodes are laid out once, in a canonical vertex order of the face, and every volume evaluates its
  basis there: the face operators are indexed by (local face, orientation, p_f), where the orientation is the vertex
  permutation between the canonical order and the volume's local face order (the reference's ind_ord,
  face.h:47-97). With the symmetric Witherden-Vincent rules this equals the reference's permutation of face nodes.
"""
from __future__ import annotations

import itertools
import math

import numpy as np

from .element import HEX, LINE, PYR, QUAD, TET, TRI, WEDGE, gauss_legendre

SQ2, SQ3, SQ6 = math.sqrt(2.0), math.sqrt(3.0), math.sqrt(6.0)

TRI_VERTS = np.array([[-1.0, -1.0 / SQ3], [1.0, -1.0 / SQ3], [0.0, 2.0 / SQ3]])
QUAD_VERTS = np.array([[-1.0, -1.0], [1.0, -1.0], [-1.0, 1.0], [1.0, 1.0]])

VERTS = {
    TET: np.array([[-1.0, -1.0 / SQ3, -1.0 / SQ6], [1.0, -1.0 / SQ3, -1.0 / SQ6], [0.0, 2.0 / SQ3, -1.0 / SQ6],
                   [0.0, 0.0, 3.0 / SQ6]]),
    WEDGE: np.array([[-1.0, -1.0 / SQ3, -1.0], [1.0, -1.0 / SQ3, -1.0], [0.0, 2.0 / SQ3, -1.0],
                     [-1.0, -1.0 / SQ3, 1.0], [1.0, -1.0 / SQ3, 1.0], [0.0, 2.0 / SQ3, 1.0]]),
    PYR: np.array([[-1.0, -1.0, -SQ2 / 5.0], [1.0, -1.0, -SQ2 / 5.0], [-1.0, 1.0, -SQ2 / 5.0],
                   [1.0, 1.0, -SQ2 / 5.0], [0.0, 0.0, 4.0 * SQ2 / 5.0]]),
    HEX: np.array([[x, y, z] for z in (-1.0, 1.0) for y in (-1.0, 1.0) for x in (-1.0, 1.0)]),
    TRI: TRI_VERTS,
    QUAD: QUAD_VERTS,
}

F_VE = {
    TET: [[2, 3, 1], [2, 3, 0], [0, 1, 3], [0, 1, 2]],
    WEDGE: [[1, 2, 4, 5], [0, 2, 3, 5], [0, 1, 3, 4], [0, 1, 2], [3, 4, 5]],
    PYR: [[0, 2, 4], [1, 3, 4], [0, 1, 4], [2, 3, 4], [0, 1, 2, 3]],
    HEX: [[0, 2, 4, 6], [1, 3, 5, 7], [0, 1, 4, 5], [2, 3, 6, 7], [0, 1, 2, 3], [4, 5, 6, 7]],
    TRI: [[1, 2], [0, 2], [0, 1]],
    QUAD: [[0, 2], [1, 3], [0, 1], [2, 3]],
}

# face orientations: vertex permutations perm with canonical face vertex m <-> local face vertex perm[m]
TRI_ORDS = [tuple(p) for p in itertools.permutations(range(3))]


def _quad_ords():
    ords = []
    for swap in (False, True):
        for sx in (1.0, -1.0):
            for sy in (1.0, -1.0):
                perm = []
                for v in QUAD_VERTS:
                    a, b = (v[1], v[0]) if swap else (v[0], v[1])
                    w = np.array([sx * a, sy * b])
                    perm.append(int(np.nonzero(np.all(np.abs(QUAD_VERTS - w) < 1e-12, axis=1))[0][0]))
                ords.append(tuple(perm))
    return ords


QUAD_ORDS = _quad_ords()          # QUAD_ORDS[0] is the identity
LINE_ORDS = [(0, 1), (1, 0)]      # the faces of 2D volumes: as is, reversed


def face_type(e_type: int, lf: int) -> int:
    nv = len(F_VE[e_type][lf])
    return LINE if nv == 2 else (TRI if nv == 3 else QUAD)


def face_ords(ftype: int):
    return LINE_ORDS if ftype == LINE else (TRI_ORDS if ftype == TRI else QUAD_ORDS)


def reference_normals_2d(e_type: int) -> np.ndarray:
    """Outward unit normals of the reference TRI per local face, in the angle form of element.c (pi/6, 5 pi/6,
    3 pi/2)."""
    if e_type != TRI:
        raise ValueError("TRI")
    return np.array([[math.cos(t), math.sin(t)] for t in (math.pi / 6.0, 5.0 * math.pi / 6.0, 1.5 * math.pi)])


def reference_normals_3d(e_type: int) -> np.ndarray:
    """Outward unit normals of the reference element per local face, in the angle form of element.c:708-780."""
    th_tet = math.atan(2.0 * SQ2)
    th_pyr = math.atan(SQ2)
    pi = math.pi
    if e_type == TET:
        t_e = [th_tet - 0.5 * pi] * 3 + [0.5 * pi]
        t_z = [pi / 6.0, 5.0 * pi / 6.0, 9.0 * pi / 6.0, 0.0]
    elif e_type == WEDGE:
        t_e = [0.0, 0.0, 0.0, 0.5 * pi, 1.5 * pi]
        t_z = [pi / 6.0, 5.0 * pi / 6.0, 9.0 * pi / 6.0, 0.0, 0.0]
    elif e_type == PYR:
        t_e = [th_pyr - 0.5 * pi] * 4 + [0.5 * pi]
        t_z = [pi, 0.0, 1.5 * pi, 0.5 * pi, 0.0]
    else:
        raise ValueError("TET, WEDGE or PYR")
    return np.array([[math.cos(e) * math.cos(z), math.cos(e) * math.sin(z), -math.sin(e)] for e, z in zip(t_e, t_z)])


# --------------------------------------------------------------------------------------------------------------------
# 1D Jacobi polynomials and Gauss-Jacobi rules
# --------------------------------------------------------------------------------------------------------------------

def jacobi_p(n: int, alpha: float, beta: float, x):
    """P_n^(alpha,beta)(x) by the three-term recurrence."""
    x = np.asarray(x, dtype=np.float64)
    p0 = np.ones_like(x)
    if n == 0:
        return p0
    p1 = 0.5 * (alpha - beta + (alpha + beta + 2.0) * x)
    for k in range(2, n + 1):
        a = alpha + beta
        c1 = 2.0 * k * (k + a) * (2.0 * k + a - 2.0)
        c2 = (2.0 * k + a - 1.0) * (alpha * alpha - beta * beta)
        c3 = (2.0 * k + a - 2.0) * (2.0 * k + a - 1.0) * (2.0 * k + a)
        c4 = 2.0 * (k + alpha - 1.0) * (k + beta - 1.0) * (2.0 * k + a)
        p0, p1 = p1, ((c2 + c3 * x) * p1 - c4 * p0) / c1
    return p1


def jacobi_dp(n: int, alpha: float, beta: float, x):
    """d/dx P_n^(alpha,beta)(x) = (n + alpha + beta + 1)/2 P_{n-1}^(alpha+1,beta+1)(x)."""
    x = np.asarray(x, dtype=np.float64)
    if n == 0:
        return np.zeros_like(x)
    return 0.5 * (n + alpha + beta + 1.0) * jacobi_p(n - 1, alpha + 1.0, beta + 1.0, x)


def gauss_jacobi(n: int, alpha: float, beta: float = 0.0):
    """Nodes and weights of the n-point Gauss rule for the weight (1-x)^alpha (1+x)^beta on [-1,1]
    (Golub-Welsch: eigen-decomposition of the Jacobi matrix, then one Newton polish of the nodes)."""
    if alpha == 0.0 and beta == 0.0:
        return gauss_legendre(n)
    k = np.arange(n, dtype=np.float64)
    ab = alpha + beta
    a = np.empty(n)
    a[0] = (beta - alpha) / (ab + 2.0)
    kk = k[1:]
    a[1:] = (beta * beta - alpha * alpha) / ((2.0 * kk + ab) * (2.0 * kk + ab + 2.0))
    kk = np.arange(1, n, dtype=np.float64)
    b = np.sqrt(4.0 * kk * (kk + alpha) * (kk + beta) * (kk + ab)
                / ((2.0 * kk + ab) ** 2 * (2.0 * kk + ab + 1.0) * (2.0 * kk + ab - 1.0)))
    T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
    x, vec = np.linalg.eigh(T)
    for _ in range(2):   # Newton on P_n^(alpha,beta)
        x = x - jacobi_p(n, alpha, beta, x) / jacobi_dp(n, alpha, beta, x)
    mu0 = 2.0 ** (ab + 1.0) * math.gamma(alpha + 1.0) * math.gamma(beta + 1.0) / math.gamma(ab + 2.0)
    # weights from the derivative formula (more accurate than the eigenvectors after the polish)
    pd = jacobi_dp(n, alpha, beta, x)
    c = (2.0 ** (ab + 1.0) * math.gamma(n + alpha + 1.0) * math.gamma(n + beta + 1.0)
         / (math.gamma(n + ab + 1.0) * math.factorial(n)))
    w = c / ((1.0 - x * x) * pd * pd)
    w *= mu0 / np.sum(w)   # exact zeroth moment
    return x, w


# --------------------------------------------------------------------------------------------------------------------
# Cubature rules on the reference elements (collapsed coordinates)
# --------------------------------------------------------------------------------------------------------------------

def _affine_from(src: np.ndarray, dst: np.ndarray):
    """A, b with dst_k = A src_k + b for the d+1 vertices of a simplex."""
    d = src.shape[1]
    S = np.hstack([src[:d + 1], np.ones((d + 1, 1))])
    M = np.linalg.solve(S, dst[:d + 1])
    return M[:d].T, M[d]


_T2 = np.array([[-1.0, -1.0], [1.0, -1.0], [-1.0, 1.0]])
_T3 = np.array([[-1.0, -1.0, -1.0], [1.0, -1.0, -1.0], [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]])


def conical_tri_rule(q: int):
    """(q^2, 2) collapsed-coordinate nodes and weights on the reference TRI (a fastest), exact to degree 2q-1."""
    xa, wa = gauss_legendre(q)
    xb, wb = gauss_jacobi(q, 1.0)
    a = np.tile(xa, q)
    bb = np.repeat(xb, q)
    w = np.tile(wa, q) * np.repeat(wb, q) * 0.5
    r = 0.5 * (1.0 + a) * (1.0 - bb) - 1.0
    s = bb
    A, b0 = _affine_from(_T2, TRI_VERTS)
    x = np.stack([r, s], axis=1) @ A.T + b0
    return x, w * abs(np.linalg.det(A))


def quad_rule(q: int):
    """(q^2, 2) GL tensor nodes (first coordinate fastest) and weights on [-1,1]^2."""
    x1, w1 = gauss_legendre(q)
    return np.stack([np.tile(x1, q), np.repeat(x1, q)], axis=1), np.tile(w1, q) * np.repeat(w1, q)


_WV = {}
_FACE_RULES = {}


def wv_rule(e_type: int, degree: int):
    """The Witherden-Vincent rule of the given degree on the reference TRI or TET: the reference's own volume
    cubature of simplices and its face cubature of 3D simplex faces (nodes_operators.c:474-516), read from
    input/nodes/{tri,tet}/WV<degree>.txt and kept in wv_rules.npz (make_wv_rules.py). Every group's barycentric
    coordinates are expanded into their orbit under the permutations of the vertices (its size is the table's), and
    mapped to the reference element as sum_i lambda_i vertex_i. Returns nodes (n, d) and weights (n,)."""
    key = (e_type, degree)
    if key not in _WV:
        import os
        name = {TRI: "tri", TET: "tet"}[e_type]
        data = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "wv_rules.npz"))
        bary, w, orbit = data[f"{name}{degree}_bary"], data[f"{name}{degree}_w"], data[f"{name}{degree}_orbit"]
        V = TRI_VERTS if e_type == TRI else VERTS[TET]
        pts, ws = [], []
        for b, wi, k in zip(bary, w, orbit):
            orb = sorted(set(itertools.permutations(b.tolist())))
            if len(orb) != k:
                raise AssertionError(f"WV{degree} orbit of {b}: {len(orb)} points, the table says {k}")
            for lam in orb:
                pts.append(np.asarray(lam) @ V)
                ws.append(wi)
        x, wt = np.array(pts), np.array(ws)
        x.setflags(write=False)
        wt.setflags(write=False)
        _WV[key] = (x, wt)
    return _WV[key]


def tri_rule(q: int):
    """The reference's TRI cubature of order p = q - 1: Witherden-Vincent of degree 2p (3, 6, 12, 16 points for
    p = 1..4)."""
    return wv_rule(TRI, 2 * (q - 1))


def quad_rule(q: int):
    """(q^2, 2) GL tensor nodes (first coordinate fastest) and weights on [-1,1]^2."""
    x1, w1 = gauss_legendre(q)
    return np.stack([np.tile(x1, q), np.repeat(x1, q)], axis=1), np.tile(w1, q) * np.repeat(w1, q)


def face_rule(ftype: int, q: int):
    """Cached (nodes, weights) of the face reference element at face order p_f = q - 1, as the reference
    integrates it (nodes_operators.c:474-516): GL with q points on LINE faces (2D) and on QUAD faces, Witherden-Vincent
    of degree 2 p_f on TRI faces (read-only arrays)."""
    key = (ftype, q)
    if key not in _FACE_RULES:
        if ftype == LINE:
            x1, w = gauss_legendre(q)
            x = x1[:, None].copy()
        else:
            x, w = tri_rule(q) if ftype == TRI else quad_rule(q)
            x, w = np.array(x), np.array(w)
        x.setflags(write=False)
        w.setflags(write=False)
        _FACE_RULES[key] = (x, w)
    return _FACE_RULES[key]


def conical_rule(e_type: int, q: int):
    """Collapsed-coordinate (conical product) Gauss-Jacobi rule with q points per direction, exact to degree
    2q-1: the exact integrations of the set-up (orthonormalisation, Bezier maps) and the PYR volume cubature."""
    if e_type == TRI:
        return conical_tri_rule(q)
    if e_type == TET:
        xa, wa = gauss_legendre(q)
        xb, wb = gauss_jacobi(q, 1.0)
        xc, wc = gauss_jacobi(q, 2.0)
        a = np.tile(xa, q * q)
        b = np.tile(np.repeat(xb, q), q)
        c = np.repeat(xc, q * q)
        w = np.tile(wa, q * q) * np.tile(np.repeat(wb, q), q) * np.repeat(wc, q * q) / 8.0
        r = 0.25 * (1.0 + a) * (1.0 - b) * (1.0 - c) - 1.0
        s = 0.5 * (1.0 + b) * (1.0 - c) - 1.0
        A, b0 = _affine_from(_T3, VERTS[TET])
        return np.stack([r, s, c], axis=1) @ A.T + b0, w * abs(np.linalg.det(A))
    if e_type == WEDGE:
        xt, wt = conical_tri_rule(q)
        xz, wz = gauss_legendre(q)
        nt = len(wt)
        x = np.hstack([np.tile(xt, (q, 1)), np.repeat(xz, nt)[:, None]])
        return x, np.tile(wt, q) * np.repeat(wz, nt)
    if e_type == PYR:
        xa, wa = gauss_legendre(q)
        xc, wc = gauss_jacobi(q, 2.0)
        a = np.tile(xa, q * q)
        b = np.tile(np.repeat(xa, q), q)
        c = np.repeat(xc, q * q)
        w = np.tile(wa, q * q) * np.tile(np.repeat(wa, q), q) * np.repeat(wc, q * q) / 4.0
        xs, ys, zs = 0.5 * a * (1.0 - c), 0.5 * b * (1.0 - c), c
        return np.stack([xs, ys, _pyr_z_to_ref(zs)], axis=1), w * (SQ2 / 2.0)
    raise ValueError("TRI, TET, WEDGE or PYR")


def volume_rule(e_type: int, q: int):
    """Volume cubature of order p = q - 1 as the reference takes it (nodes_operators.c:474-516): Witherden-Vincent
    of degree 2p on TRI and TET; on the WEDGE the product of that TRI rule and GL with q points (the reference builds
    WEDGE operators from their TRI and LINE factors, element_operators_tp.c); on the PYR the conical Gauss-Jacobi
    rule with q points per direction (exact to degree 2p + 1). The reference's own PYR choice, GJW, stops at
    compute_cub_c_type (nodes_operators.c:589-609), which has no case for it."""
    if e_type in (TRI, TET):
        x, w = wv_rule(e_type, 2 * (q - 1))
        return np.array(x), np.array(w)
    if e_type == WEDGE:
        xt, wt = tri_rule(q)
        xz, wz = gauss_legendre(q)
        nt = len(wt)
        x = np.hstack([np.tile(xt, (q, 1)), np.repeat(xz, nt)[:, None]])
        return x, np.tile(wt, q) * np.repeat(wz, nt)
    if e_type == PYR:
        return conical_rule(PYR, q)
    raise ValueError("TRI, TET, WEDGE or PYR")


def _pyr_z_to_ref(z):
    """Standard pyramid (base z = -1, apex z = 1) -> reference pyramid height coordinate."""
    return (z + 1.0) * (SQ2 / 2.0) - SQ2 / 5.0


def _pyr_ref_to_std(x):
    return x[:, 0], x[:, 1], (x[:, 2] + SQ2 / 5.0) * SQ2 - 1.0


# --------------------------------------------------------------------------------------------------------------------
# Orthonormal bases (values and reference-coordinate gradients)
# --------------------------------------------------------------------------------------------------------------------

def _leg(n, x):
    return jacobi_p(n, 0.0, 0.0, x), jacobi_dp(n, 0.0, 0.0, x)


def _raw_basis(e_type: int, p: int, x: np.ndarray):
    """Unnormalised spanning functions of the solution space at points x (n, 3): values (n, m), gradients
    (3, n, m)."""
    cols, grads = [], []
    if e_type == TRI:
        return _raw_tri(p, x)
    if e_type == TET:
        for tot in range(p + 1):
            for a in range(tot, -1, -1):
                for b in range(tot - a, -1, -1):
                    c = tot - a - b
                    (pa, da), (pb, db), (pc, dc) = _leg(a, x[:, 0]), _leg(b, x[:, 1]), _leg(c, x[:, 2])
                    cols.append(pa * pb * pc)
                    grads.append([da * pb * pc, pa * db * pc, pa * pb * dc])
    elif e_type == WEDGE:
        for c in range(p + 1):
            for tot in range(p + 1):
                for a in range(tot, -1, -1):
                    b = tot - a
                    (pa, da), (pb, db), (pc, dc) = _leg(a, x[:, 0]), _leg(b, x[:, 1]), _leg(c, x[:, 2])
                    cols.append(pa * pb * pc)
                    grads.append([da * pb * pc, pa * db * pc, pa * pb * dc])
    elif e_type == PYR:
        xs, ys, zs = _pyr_ref_to_std(x)
        om = 1.0 - zs
        a = 2.0 * xs / om
        b = 2.0 * ys / om
        for m in range(p + 1):
            for i in range(m + 1):
                for j in range(m + 1):
                    if max(i, j) != m:
                        continue
                    for k in range(p - m + 1):
                        (pa, da), (pb, db) = _leg(i, a), _leg(j, b)
                        jk = jacobi_p(k, 2.0 * m + 2.0, 0.0, zs)
                        djk = jacobi_dp(k, 2.0 * m + 2.0, 0.0, zs)
                        h = (0.5 * om) ** m
                        dh = -0.5 * m * (0.5 * om) ** (m - 1) if m > 0 else np.zeros_like(zs)
                        C = h * jk
                        dC = dh * jk + h * djk
                        cols.append(pa * pb * C)
                        gx = da * pb * C * 2.0 / om
                        gy = pa * db * C * 2.0 / om
                        gz = (da * pb * a + pa * db * b) * C / om + pa * pb * dC
                        grads.append([gx, gy, gz * SQ2])   # d z_std / d z_ref = sqrt2
    else:
        raise ValueError("TET, WEDGE or PYR")
    V = np.stack(cols, axis=1)
    G = np.stack([np.stack([g[k] for g in grads], axis=1) for k in range(3)])
    return V, G


def _raw_tri(p: int, x: np.ndarray):
    """P_a(x) P_b(y), a + b <= p, in the order of the WEDGE's inner index: values (n, m), gradients (2, n, m)."""
    cols, gx, gy = [], [], []
    for tot in range(p + 1):
        for a in range(tot, -1, -1):
            b = tot - a
            (pa, da), (pb, db) = _leg(a, x[:, 0]), _leg(b, x[:, 1])
            cols.append(pa * pb)
            gx.append(da * pb)
            gy.append(pa * db)
    return np.stack(cols, axis=1), np.stack([np.stack(gx, axis=1), np.stack(gy, axis=1)])


def _orthonormaliser(V: np.ndarray, w: np.ndarray) -> np.ndarray:
    """C with (V C)^T diag(w) (V C) = I (QR, then one re-orthogonalisation pass)."""
    _, R = np.linalg.qr(np.sqrt(w)[:, None] * V)
    Cm = np.linalg.inv(R)
    _, R2 = np.linalg.qr(np.sqrt(w)[:, None] * (V @ Cm))
    return Cm @ np.linalg.inv(R2)


def n_basis(e_type: int, p: int) -> int:
    if e_type == TRI:
        return (p + 1) * (p + 2) // 2
    if e_type == TET:
        return (p + 1) * (p + 2) * (p + 3) // 6
    if e_type == WEDGE:
        return (p + 1) * (p + 1) * (p + 2) // 2
    if e_type == PYR:
        return (p + 1) * (p + 2) * (2 * p + 3) // 6
    raise ValueError("TET, WEDGE or PYR")


class DenseOperatorSet:
    """Operators of one (TET | WEDGE | PYR, p) group for the dense-operator kernels and the oracle.

    cv0_vs_vc (n_vc x n_vs), cv1_vs_vc (3 x n_vc x n_vs) in reference coordinates, w_vc (n_vc); face operators
    cv0_vs_fc(lf, ord, q_f) (n_fc x n_vs) at the canonical face nodes of face_rule(face_type, q_f)."""

    dense = True

    def __init__(self, e_type: int, p: int):
        if e_type not in (TRI, TET, WEDGE, PYR):
            raise ValueError("TRI, TET, WEDGE or PYR")
        if not 1 <= p <= 4:
            raise ValueError("p in 1..4")
        self.e_type, self.p, self.d, self.q = e_type, p, (2 if e_type == TRI else 3), p + 1
        self.n_vs = n_basis(e_type, p)
        self.x_vc, self.w_vc = volume_rule(e_type, p + 1)
        self.n_vc = len(self.w_vc)
        self.n_lf = len(F_VE[e_type])
        self.normals_ref = reference_normals_2d(e_type) if e_type == TRI else reference_normals_3d(e_type)
        if e_type == WEDGE:
            # the product of an orthonormal TRI basis and the normalised Legendre polynomials, so that every
            # volume operator is a Kronecker product (prism_factors)
            xt, wt = conical_tri_rule(p + 2)
            Vt, _ = _raw_tri(p, xt)
            self._Ct = _orthonormaliser(Vt, wt)
            self._Cl = np.diag([math.sqrt(0.5 * (2 * c + 1)) for c in range(p + 1)])
            self._C = np.kron(self._Cl, self._Ct)
        else:
            # orthonormalise the spanning functions with a rule exact for their products
            xg, wg = conical_rule(e_type, p + 2)
            Vg, _ = _raw_basis(e_type, p, xg)
            if Vg.shape[1] != self.n_vs:
                raise AssertionError("basis dimension")
            self._C = _orthonormaliser(Vg, wg)
        self._cache = {}
        V, G = self.basis(self.x_vc)
        self._cv0 = V
        self._cv1 = G

    def basis(self, x):
        V, G = _raw_basis(self.e_type, self.p, np.asarray(x, dtype=np.float64))
        return V @ self._C, np.stack([G[k] @ self._C for k in range(self.d)])

    def prism_factors(self):
        """WEDGE only: (tri_cv0 (n_tvc x n_tvs), tri_cv1 (2 x n_tvc x n_tvs), line_cv0, line_cv1 (q x q)) with
        cv0_vs_vc = kron(line_cv0, tri_cv0), cv1_vs_vc[0/1] = kron(line_cv0, tri_cv1[0/1]) and
        cv1_vs_vc[2] = kron(line_cv1, tri_cv0) (basis index c * n_tvs + t, node index rz * n_tvc + rt)."""
        if self.e_type != WEDGE:
            raise ValueError("WEDGE only")
        q = self.q
        xt, _ = tri_rule(q)
        Vt, Gt = _raw_tri(self.p, xt)
        xz, _ = gauss_legendre(q)
        Vl = np.stack([jacobi_p(c, 0.0, 0.0, xz) for c in range(q)], axis=1)
        Dl = np.stack([jacobi_dp(c, 0.0, 0.0, xz) for c in range(q)], axis=1)
        return (Vt @ self._Ct, np.stack([Gt[0] @ self._Ct, Gt[1] @ self._Ct]), Vl @ self._Cl, Dl @ self._Cl)

    def _bezier_maps(self):
        if "bez" not in self._cache:
            x, w = conical_rule(self.e_type, self.p + 2)
            B = bezier_basis(self.e_type, self.p, x)
            if B.shape[1] != self.n_vs:
                raise AssertionError("Bezier basis dimension")
            S_ = self.basis(x)[0]
            sb = np.linalg.lstsq(B, S_, rcond=None)[0]          # solution basis in the Bezier basis: S = B sb
            if np.abs(B @ sb - S_).max() > 1e-10 * max(1.0, np.abs(S_).max()):
                raise AssertionError("the Bezier functions do not span the solution space")
            self._cache["bez"] = (sb, np.linalg.inv(sb))
        return self._cache["bez"]

    def ccSB0_vs_vs(self):
        """Solution-basis coefficients -> Bezier coefficients (the reference's ccSB0_vs_vs)."""
        return self._bezier_maps()[0]

    def ccBS0_vs_vs(self):
        """Bezier coefficients -> solution-basis coefficients (ccBS0_vs_vs)."""
        return self._bezier_maps()[1]

    def cv0_vs_vc(self):
        return self._cv0

    def cv1_vs_vc(self, dim: int):
        return self._cv1[dim]

    def tw1_vt_vc(self, dim: int):
        return self._cv1[dim].T * self.w_vc[None, :]

    def mass(self):
        return self._cv0.T @ (self.w_vc[:, None] * self._cv0)

    def face_type(self, lf: int) -> int:
        return face_type(self.e_type, lf)

    def n_ords(self, lf: int) -> int:
        return len(face_ords(self.face_type(lf)))

    def face_points(self, lf: int, ord_: int, q_f: int):
        """Reference coordinates of the canonical face nodes of local face lf seen with orientation ord_."""
        ft = self.face_type(lf)
        xi, _ = face_rule(ft, q_f)
        perm = face_ords(ft)[ord_]
        R = VERTS[self.e_type][F_VE[self.e_type][lf]]
        return face_shape(ft, xi) @ R[list(perm)]

    def cv0_vs_fc(self, lf: int, ord_: int, q_f: int):
        key = (lf, ord_, q_f)
        if key not in self._cache:
            self._cache[key] = self.basis(self.face_points(lf, ord_, q_f))[0]
        return self._cache[key]

    def w_fc(self, lf: int, q_f: int):
        return face_rule(self.face_type(lf), q_f)[1]


def _bern(n: int, k: int, x):
    """1D Bernstein polynomial C(n, k) ((1 + x) / 2)^k ((1 - x) / 2)^(n - k) on [-1, 1]."""
    return math.comb(n, k) * (0.5 * (1.0 + x)) ** k * (0.5 * (1.0 - x)) ** (n - k)


def bezier_basis(e_type: int, p: int, x: np.ndarray) -> np.ndarray:
    """The reference's Bezier basis at points x (n, d) (bases.c:570-760): the Bernstein polynomials of the
    barycentric coordinates on TRI and TET (constructor_basis_si_bezier writes the same functions in collapsed
    coordinates), the TRI x LINE product on WEDGE, and on PYR the products B^{p-k}_i(a) B^{p-k}_j(b) B^p_k(c) of the
    collapsed coordinates (constructor_basis_pyr_bezier). The limiter only uses their set, not their order."""
    x = np.asarray(x, dtype=np.float64)
    cols = []
    if e_type in (TRI, TET):
        V = VERTS[e_type]
        d = V.shape[1]
        T = np.vstack([V.T, np.ones(d + 1)])
        lam = np.linalg.solve(T, np.vstack([x.T, np.ones(len(x))])).T          # barycentric coordinates
        import itertools
        for alpha in itertools.product(range(p + 1), repeat=d + 1):
            if sum(alpha) != p:
                continue
            c = math.factorial(p)
            val = np.ones(len(x))
            for m, a in enumerate(alpha):
                c //= math.factorial(a)
                val = val * lam[:, m] ** a
            cols.append(c * val)
    elif e_type == WEDGE:
        tri = bezier_basis(TRI, p, x[:, :2])
        for k in range(p + 1):
            lk = _bern(p, k, x[:, 2])
            for t in range(tri.shape[1]):
                cols.append(tri[:, t] * lk)
    elif e_type == PYR:
        xs, ys, zs = _pyr_ref_to_std(x)
        om = 1.0 - zs
        a, b = 2.0 * xs / om, 2.0 * ys / om
        for i in range(p + 1):
            for j in range(p + 1):
                for k in range(p - max(i, j) + 1):
                    cols.append(_bern(p - k, i, a) * _bern(p - k, j, b) * _bern(p, k, zs))
    else:
        raise ValueError("TRI, TET, WEDGE or PYR")
    return np.stack(cols, axis=1)


def face_shape(ftype: int, xi: np.ndarray) -> np.ndarray:
    """(n, n_vertices) shape functions of the face reference element at xi: barycentric coordinates on the TRI,
    bilinear in tensor vertex order on the QUAD, linear on the LINE."""
    if ftype == LINE:
        t = xi[:, 0]
        return np.stack([0.5 * (1.0 - t), 0.5 * (1.0 + t)], axis=1)
    if ftype == TRI:
        T = np.vstack([TRI_VERTS.T, np.ones(3)])
        lam = np.linalg.solve(T, np.vstack([xi.T, np.ones(len(xi))]))
        return lam.T
    x, y = xi[:, 0], xi[:, 1]
    return np.stack([0.25 * (1 - x) * (1 - y), 0.25 * (1 + x) * (1 - y), 0.25 * (1 - x) * (1 + y),
                     0.25 * (1 + x) * (1 + y)], axis=1)
