"""TP element layer pinned against the reference's own unit-test golden data (tests/golden/, extracted from
input/testing/unit/{operators,nodes}/*.data by tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from dpgsolver_gb300.host import element as el

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_unit_data.json")))
EPS = 1e-15  # definitions_tol.h:23, the tolerance of test_unit_operators_tp.c


@pytest.mark.parametrize("name", ["quad", "hex"])
def test_tp_op_std_assembly(name):
    """op_std = kron of ops_tp with the first direction fastest (test_unit_operators_tp.c:88-124)."""
    g = GOLDEN["operators_tp"][name]
    ops = [np.array(o) for o in g["ops_tp"]]
    op_std = el.kron_tp(ops)
    ref = np.array(g["op_std"])
    # the data file prints op_std with 4 significant digits
    assert op_std.shape == ref.shape
    assert np.max(np.abs(op_std - ref)) < 5e-5


@pytest.mark.parametrize("name", ["quad", "hex"])
def test_tp_apply_sum_factorised(name):
    """c = op_std . b, applied direction by direction (constructor_mm_tp_NN1C_const_Multiarray_T,
    multiarray_constructors_T.c:448-540; golden vectors quad_c/hex_c)."""
    g = GOLDEN["operators_tp"][name]
    ops = [np.array(o) for o in g["ops_tp"]]
    b = np.array(g["b"])
    c_ref = np.array(g["c"])
    # sum-factorised apply: reshape with the first direction fastest
    d = len(ops)
    in_ext = [o.shape[1] for o in ops]
    cols = []
    for col in range(b.shape[1]):
        x = b[:, col].reshape(in_ext[::-1])  # (t, s, r) C-order == r fastest
        for k, op in enumerate(ops):
            axis = d - 1 - k
            x = np.moveaxis(np.tensordot(op, x, axes=([1], [axis])), 0, axis)
        cols.append(x.reshape(-1))
    c = np.stack(cols, axis=1)
    assert np.max(np.abs(c - c_ref)) <= 10 * EPS * np.max(np.abs(c_ref))
    # the same result through the assembled dense operator
    c2 = el.kron_tp(ops) @ b
    assert np.max(np.abs(c2 - c_ref)) <= 10 * EPS * np.max(np.abs(c_ref))


@pytest.mark.parametrize("key", ["Nodes_d1_p3_GLoL", "Nodes_d1_p3_GLe", "Nodes_d2_p4_GLoL", "Nodes_d2_p4_GLe",
                                 "Nodes_d3_p3_GLoL", "Nodes_d3_p3_GLe", "Nodes_d2_p4_EQ", "Nodes_d3_p3_EQ"])
def test_tp_nodes_and_weights(key):
    g = GOLDEN["nodes_tp"][key]
    d, p, kind = g["d"], g["p"], g["type"]
    q = p + 1
    if kind == "GLoL":
        x, w = el.gauss_lobatto(q)
    elif kind == "GLe":
        x, w = el.gauss_legendre(q)
    else:
        x, w = el.equispaced(q), None
    rst = el.tp_nodes(x, d)
    assert np.max(np.abs(rst - np.array(g["rst"]))) <= 2e-16 * 4
    if w is not None:
        wt = el.tp_weights(w, d)
        assert np.max(np.abs(wt - np.array(g["w"]))) <= 2e-16 * 8


@pytest.mark.parametrize("key,q,face_d", [("line_3", 3, 1), ("line_4", 4, 1), ("quad_9", 3, 2), ("quad_16", 4, 2)])
def test_face_node_correspondence(key, q, face_d):
    """nc_fc permutations per ind_ord (test_unit_nodes.c:62-89, nodes_correspondence.data)."""
    ref = GOLDEN["nodes_correspondence"][key]
    assert el.face_node_permutations(q, face_d) == ref


def test_reference_normals_match_element_c():
    n = el.reference_normals(el.QUAD)
    assert np.allclose(n, [[-1, 0], [1, 0], [0, -1], [0, 1]], atol=1e-15)
    assert n[0, 1] != 0.0  # sin(pi) round-off kept, as element.c computes it
    n3 = el.reference_normals(el.HEX)
    assert np.allclose(n3, [[-1, 0, 0], [1, 0, 0], [0, -1, 0], [0, 1, 0], [0, 0, -1], [0, 0, 1]], atol=1e-15)


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_operator_identities(p):
    """Identities the GB300 formulation relies on: cv1 = Dgl B, cv0_fc = l_gl B, and B invertible."""
    ops = el.TPOperatorSet(el.HEX, p)
    B = ops.cv0_1d
    Binv = np.linalg.inv(B)
    Dgl = el.lagrange_derivative_matrix(ops.x_vc, ops.x_vc)
    assert np.max(np.abs(Dgl @ B - ops.cv1_1d)) < 1e-13
    lgl = el.lagrange_matrix(ops.x_vc, np.array([-1.0, 1.0]))
    assert np.max(np.abs(lgl @ B - ops.cv0_bnd_1d)) < 1e-13
    assert np.linalg.cond(B) < 50
    assert np.max(np.abs(ops.ccBS0_1d @ ops.ccSB0_1d - np.eye(p + 1))) < 1e-13
    # partition of unity of the Bezier basis: constants map to constants
    assert np.allclose(ops.ccSB0_1d.sum(axis=1), 1.0)
    assert np.max(np.abs(Binv @ B - np.eye(p + 1))) < 1e-13
