"""Reference-element data for tensor-product (QUAD/HEX) DG elements.

This is the caller-side set-up that the reference builds in its element layer
(src/element/*.c, src/simulation/solvers/element_solver.c) and hands to the
explicit residual as read-only operators.  Nothing here runs per time step.

Conventions mirrored from the reference:

* Solution basis: Lagrange on Gauss-Lobatto-Legendre (GLL) nodes, ``interp_tp GLL``
  (input/testing/control_files/euler/periodic_vortex/*.ctrl), so the solution
  coefficients are nodal values.
* Volume and face cubature on TP elements: Gauss-Legendre (GL) with p+1 points per
  direction (cubature order p_c_x*p = 2p halved for GL, element/nodes_operators.c:314-356,
  589-610; defaults simulation.c:494-500).
* Tensor-product node ordering with the first reference coordinate fastest, and
  std operators formed as Kronecker products of 1D operators in that order
  (element/element_operators_tp.c; pinned by input/testing/unit/operators/operators_tp.data).
* Local face numbering QUAD: 0 r=-1, 1 r=+1, 2 s=-1, 3 s=+1; HEX adds 4 t=-1, 5 t=+1,
  with reference normals from element/element.c:708-780.
"""
from __future__ import annotations

import math
import numpy as np

# Element type codes (element/definitions_elements.h:32-39).
LINE, TRI, QUAD, TET, HEX, WEDGE, PYR = 1, 2, 3, 4, 5, 6, 7


# --------------------------------------------------------------------------------------------------------------------
# 1D nodes
# --------------------------------------------------------------------------------------------------------------------

def _legendre_and_derivative(n: int, x: np.ndarray):
    """P_n(x) and P_n'(x) by the three-term recurrence."""
    p0 = np.ones_like(x)
    if n == 0:
        return p0, np.zeros_like(x)
    p1 = x.copy()
    for k in range(2, n + 1):
        p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
    with np.errstate(divide="ignore", invalid="ignore"):
        dp = n * (x * p1 - p0) / (x * x - 1.0)  # not used at x = +-1
    return p1, dp


def gauss_legendre(q: int):
    """Gauss-Legendre nodes/weights on [-1,1], ascending (reference node type "GL")."""
    x, w = np.polynomial.legendre.leggauss(q)
    # One Newton polish on P_q for the last ulp; weights from the standard formula.
    p, dp = _legendre_and_derivative(q, x)
    x = x - p / dp
    p, dp = _legendre_and_derivative(q, x)
    w = 2.0 / ((1.0 - x * x) * dp * dp)
    x = 0.5 * (x - x[::-1])  # exact symmetry
    w = 0.5 * (w + w[::-1])
    return x, w


def gauss_lobatto(q: int):
    """Gauss-Lobatto-Legendre nodes/weights on [-1,1], ascending (reference node type "GLL")."""
    if q < 2:
        raise ValueError("GLL needs at least 2 nodes")
    n = q - 1
    # Interior nodes: roots of P_n'. Start from Chebyshev-Gauss-Lobatto points and Newton-iterate on
    # (1-x^2) P_n'(x), whose derivative is -n(n+1) P_n(x).
    x = -np.cos(np.pi * np.arange(q) / n)
    for _ in range(100):
        inner = x[1:-1]
        pi, dpi = _legendre_and_derivative(n, inner)
        f = (1.0 - inner * inner) * dpi
        fp = -n * (n + 1) * pi
        dx = f / fp
        x[1:-1] = inner - dx
        if np.max(np.abs(dx), initial=0.0) < 1e-17:
            break
    x[0], x[-1] = -1.0, 1.0
    pn, _ = _legendre_and_derivative(n, x)
    w = 2.0 / (n * (n + 1) * pn * pn)
    x = 0.5 * (x - x[::-1])
    w = 0.5 * (w + w[::-1])
    return x, w


def equispaced(q: int):
    return np.linspace(-1.0, 1.0, q)


def tp_nodes(x1: np.ndarray, d: int) -> np.ndarray:
    """TP node coordinates (n, d), first coordinate fastest (element/nodes.c TP ordering)."""
    q = len(x1)
    if d == 1:
        return x1.reshape(q, 1).copy()
    if d == 2:
        r, s = np.meshgrid(x1, x1, indexing="xy")
        return np.stack([r.ravel(), s.ravel()], axis=1)
    r, s, t = np.meshgrid(x1, x1, x1, indexing="ij")
    # want index i + q*j + q^2*k  with coords (x_i, x_j, x_k)
    r = np.transpose(r, (2, 1, 0)).ravel()
    s = np.transpose(s, (2, 1, 0)).ravel()
    t = np.transpose(t, (2, 1, 0)).ravel()
    return np.stack([r, s, t], axis=1)


def tp_weights(w1: np.ndarray, d: int) -> np.ndarray:
    w = w1.copy()
    for _ in range(d - 1):
        w = np.kron(w1, w)
    return w


# --------------------------------------------------------------------------------------------------------------------
# 1D bases
# --------------------------------------------------------------------------------------------------------------------

def lagrange_matrix(xn: np.ndarray, x: np.ndarray) -> np.ndarray:
    """L[m, i] = l_i(x_m) for the Lagrange basis on nodes xn (exact 0/1 at the nodes)."""
    xn = np.asarray(xn, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    q = len(xn)
    L = np.empty((len(x), q))
    for i in range(q):
        num = np.ones(len(x))
        den = 1.0
        for k in range(q):
            if k == i:
                continue
            num = num * (x - xn[k])
            den *= xn[i] - xn[k]
        L[:, i] = num / den
    for m in range(len(x)):
        hit = np.nonzero(x[m] == xn)[0]
        if len(hit):
            L[m, :] = 0.0
            L[m, hit[0]] = 1.0
    return L


def lagrange_derivative_matrix(xn: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Dm[m, i] = l_i'(x_m)."""
    xn = np.asarray(xn, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    q = len(xn)
    D = np.zeros((len(x), q))
    for i in range(q):
        den = 1.0
        for k in range(q):
            if k != i:
                den *= xn[i] - xn[k]
        for j in range(q):
            if j == i:
                continue
            term = np.ones(len(x))
            for k in range(q):
                if k != i and k != j:
                    term = term * (x - xn[k])
            D[:, i] += term
        D[:, i] /= den
    return D


def bernstein_matrix(p: int, x: np.ndarray) -> np.ndarray:
    """Bm[m, k] = b_{k,p}(x_m), Bernstein polynomials of degree p on [-1,1]."""
    t = 0.5 * (np.asarray(x, dtype=np.float64) + 1.0)
    Bm = np.empty((len(t), p + 1))
    for k in range(p + 1):
        Bm[:, k] = math.comb(p, k) * t ** k * (1.0 - t) ** (p - k)
    return Bm


# --------------------------------------------------------------------------------------------------------------------
# TP assembly
# --------------------------------------------------------------------------------------------------------------------

def kron_tp(ops_1d):
    """std operator from 1D factors [op_r, op_s, (op_t)], first reference coordinate fastest.

    Matches the reference's construction of op_std from ops_tp (element_operators_tp.c) as pinned by
    operators_tp.data: quad_op_std = kron(ops[1], ops[0]).
    """
    out = ops_1d[0]
    for op in ops_1d[1:]:
        out = np.kron(op, out)
    return out


def reference_normals(e_type: int) -> np.ndarray:
    """Reference-element outward unit normals per local face, as element/element.c:708-780 computes
    them (including the cos/sin round-off of the angle form)."""
    if e_type == QUAD:
        t_e = [0.0, 0.0, 0.0, 0.0]
        t_z = [math.pi, 0.0, 1.5 * math.pi, 0.5 * math.pi]
        d = 2
    elif e_type == HEX:
        t_e = [0.0, 0.0, 0.0, 0.0, 0.5 * math.pi, 1.5 * math.pi]
        t_z = [math.pi, 0.0, 1.5 * math.pi, 0.5 * math.pi, 0.0, math.pi]
        d = 3
    else:
        raise ValueError("unsupported element type")
    n = []
    for te, tz in zip(t_e, t_z):
        row = [math.cos(te) * math.cos(tz), math.cos(te) * math.sin(tz)]
        if d > 2:
            row.append(-math.sin(te))
        n.append(row)
    return np.array(n)


def face_tangential_dirs(d: int, lf: int):
    """Reference directions that parametrise local face lf (first listed = fastest face coordinate)."""
    normal_dir = lf // 2
    return [k for k in range(d) if k != normal_dir]


class TPOperatorSet:
    """1D factors and std (dense) operators of one (element type, p) group.

    Names follow the reference's operator naming (element/element_operators.h:21-89):
    cv0_vs_vc: solution coefficients -> values at volume cubature nodes; cv1: first derivative;
    tw1_vt_vc[d] = (cv1_vt_vc[d])^T diag(w_vc) (element_operators.c:670-720); cv0_vs_fc[lf],
    tw0_vt_fc[lf] = (cv0_vt_fc[lf])^T diag(w_fc); ccSB0/ccBS0: Lagrange <-> Bezier coefficients.
    """

    def __init__(self, e_type: int, p: int):
        if e_type not in (QUAD, HEX):
            raise ValueError("TPOperatorSet supports QUAD and HEX")
        if p < 1:
            raise ValueError("p >= 1 required")
        self.e_type = e_type
        self.d = 2 if e_type == QUAD else 3
        self.p = p
        q = p + 1
        self.q = q
        self.x_vs, _ = gauss_lobatto(q)
        self.x_vc, self.w_vc_1d = gauss_legendre(q)
        self.x_fc, self.w_fc_1d = self.x_vc, self.w_vc_1d
        # 1D factors
        self.cv0_1d = lagrange_matrix(self.x_vs, self.x_vc)              # (q_c x q_s)
        self.cv1_1d = lagrange_derivative_matrix(self.x_vs, self.x_vc)   # (q_c x q_s)
        self.cv0_bnd_1d = lagrange_matrix(self.x_vs, np.array([-1.0, 1.0]))  # (2 x q_s)
        Bm = bernstein_matrix(p, self.x_vs)                                  # values of Bernstein at GLL
        self.ccBS0_1d = Bm                       # Bezier coef -> Lagrange coef (nodal values)
        self.ccSB0_1d = np.linalg.inv(Bm)        # Lagrange coef -> Bezier coef
        d = self.d
        self.n_vs = q ** d
        self.n_vc = q ** d
        self.n_fc = q ** (d - 1)
        self.n_lf = 2 * d
        self.w_vc = tp_weights(self.w_vc_1d, d)
        self.w_fc = tp_weights(self.w_fc_1d, d - 1)
        self.normals_ref = reference_normals(e_type)

    # dense operators (the reference's op_std, used by the oracle) ---------------------------------------------------
    def cv0_vs_vc(self):
        return kron_tp([self.cv0_1d] * self.d)

    def cv1_vs_vc(self, dim: int):
        ops = [self.cv0_1d] * self.d
        ops = list(ops)
        ops[dim] = self.cv1_1d
        return kron_tp(ops)

    def tw1_vt_vc(self, dim: int):
        return self.cv1_vs_vc(dim).T * self.w_vc[None, :]

    def cv0_vs_fc(self, lf: int):
        d = self.d
        nd = lf // 2
        side = lf % 2
        ops = []
        for k in range(d):
            if k == nd:
                ops.append(self.cv0_bnd_1d[side:side + 1, :])
            else:
                ops.append(self.cv0_1d)
        return kron_tp(ops)

    def tw0_vt_fc(self, lf: int):
        return self.cv0_vs_fc(lf).T * self.w_fc[None, :]

    def ccSB0_vs_vs(self):
        return kron_tp([self.ccSB0_1d] * self.d)

    def ccBS0_vs_vs(self):
        return kron_tp([self.ccBS0_1d] * self.d)

    def face_node_ref_coords(self, lf: int) -> np.ndarray:
        """Volume reference coordinates of the face cubature nodes of local face lf, face-node order."""
        d = self.d
        nd = lf // 2
        val = -1.0 if lf % 2 == 0 else 1.0
        tdirs = face_tangential_dirs(d, lf)
        fn = tp_nodes(self.x_fc, d - 1)
        out = np.empty((self.n_fc, d))
        out[:, nd] = val
        for a, k in enumerate(tdirs):
            out[:, k] = fn[:, a]
        return out


def face_node_permutations(q: int, face_d: int):
    """Face-node correspondence permutations indexed by the reference's ``ind_ord``.

    LINE faces (face_d = 1): 0 identity, 1 reversed. QUAD faces (face_d = 2), node index a + q*b with
    ind_ord 0..7 = identity, flip a, flip b, flip both, transpose, and the transposes composed with the flips,
    in the order pinned by input/testing/unit/nodes/nodes_correspondence.data (test_unit_nodes.c:62-89).
    Entry i of a permutation is the node index on the other side that matches node i.
    """
    if face_d == 1:
        return [list(range(q)), list(range(q - 1, -1, -1))]
    if face_d != 2:
        raise ValueError("face_d must be 1 or 2")
    r = q - 1
    maps = [
        lambda a, b: (a, b),
        lambda a, b: (r - a, b),
        lambda a, b: (a, r - b),
        lambda a, b: (r - a, r - b),
        lambda a, b: (b, a),
        lambda a, b: (r - b, a),
        lambda a, b: (b, r - a),
        lambda a, b: (r - b, r - a),
    ]
    perms = []
    for f in maps:
        perm = []
        for i in range(q * q):
            a, b = i % q, i // q
            a2, b2 = f(a, b)
            perm.append(a2 + q * b2)
        perms.append(perm)
    return perms


def face_operators(ops: "TPOperatorSet", q_f: int):
    """cv0_vs_fc[lf] and tw0_vt_fc[lf] of a (type, p) volume at the face cubature of order p_f = q_f - 1
    (the reference's cv0_vs_fc[lf][p_f][p_v], tw0_vt_fc = cv0^T diag(w_fc); compute_face_rlhs_T.c:51-81):
    GL with q_f points per tangential direction; q_f >= ops.q (p_f = max(p_L, p_R), face_solver.c:123-132)."""
    if q_f < ops.q:
        raise ValueError("face order below the volume order")
    x_f, w_f1 = gauss_legendre(q_f)
    d = ops.d
    tang = lagrange_matrix(ops.x_vs, x_f)             # (q_f x q_v)
    w_fc = tp_weights(w_f1, d - 1)
    cv0, tw0 = [], []
    for lf in range(2 * d):
        nd, side = lf // 2, lf % 2
        one_d = [ops.cv0_bnd_1d[side:side + 1, :] if k == nd else tang for k in range(d)]
        c = kron_tp(one_d)
        cv0.append(c)
        tw0.append(c.T * w_fc[None, :])
    return cv0, tw0, w_fc
