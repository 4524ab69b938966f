"""The mesh reader and connectivity (include/dgpu_mesh.h) against the reference's mesh integration fixtures, and
meshes read from files through the oracle.

Golden: the three gmsh files of input/testing/integration/mesh with their .msh.data (Mesh_Data, Mesh_Connectivity,
Mesh_Vertices as test_integration_mesh.c:71-150 compares them), extracted by tests/golden/make_mesh_golden.py:
a periodic QUAD mesh, a mixed TRI/QUAD mesh with straight and curved boundaries, and a QUAD mesh with
a periodic pair and a reflected periodic pair. Every integer field must match exactly.

Written meshes: structured boxes whose volumes have random local frames, so that neighbours see their common face
in any of the reference's orderings; the residual on such a mesh must equal the residual on the same mesh with
aligned frames at every physical solution node (the face permutations are what makes them agree).
"""
import json
import os

import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import gmsh as G
from dpgsolver_gb300.host import problem as P

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_mesh_data.json")))


def _lists(a):
    return [list(map(int, x)) for x in a]


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_reader_and_connectivity_match_reference_fixture(tmp_path, name):
    g = GOLDEN[name]
    path = tmp_path / (name + ".msh")
    path.write_text(g["msh"])
    m = G.GmshMesh(path, g["d"])
    ex = g["expected"]
    assert list(m.elem_per_dim) == ex["elem_per_dim"]
    assert np.max(np.abs(m.nodes - np.array(ex["nodes"]))) < 1e-12   # the fixture prints 13 digits
    assert list(m.elem_types) == ex["elem_types"]
    assert m.elem_tags.tolist() == ex["elem_tags"]
    assert _lists(m.node_nums) == ex["node_nums"]
    if "periodic_corr" in ex:
        assert m.periodic_corr.tolist() == ex["periodic_corr"]
    assert _lists(m.v_to_v) == ex["v_to_v"]
    assert _lists(m.v_to_lf) == ex["v_to_lf"]
    if "v_to_lf_wp" in ex:
        assert _lists(m.v_to_lf_wp) == ex["v_to_lf_wp"]
    else:
        assert m.v_to_lf_wp is None
    assert list(m.ve_curved) == ex["ve_curved"]
    assert list(m.ve_boundary) == ex["ve_boundary"]
    assert _lists(m.ve_bc) == ex["ve_bc"]


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_face_list_follows_connectivity(tmp_path, name):
    """constructor_Faces: every local face of every volume in exactly one face, side 1 its neighbour, boundary faces
    carrying the BC code and no ordering, interior faces an ordering index in the reference's permutation list."""
    g = GOLDEN[name]
    path = tmp_path / (name + ".msh")
    path.write_text(g["msh"])
    m = G.GmshMesh(path, g["d"])
    seen = set()
    for f in range(m.n_faces):
        v, lf = m.face_vol[f, 0], m.face_lf[f, 0]
        seen.add((v, lf))
        if m.face_vol[f, 1] >= 0:
            w, lw = m.face_vol[f, 1], m.face_lf[f, 1]
            seen.add((w, lw))
            assert m.v_to_v[v][lf] == w and m.v_to_lf[v][lf] == lw and m.face_bc[f] == -1
            assert 0 <= m.face_ord[f, 0] and 0 <= m.face_ord[f, 1]
        else:
            assert m.face_bc[f] == m.v_to_lf[v][lf] > 10000 and m.face_ord[f].tolist() == [-1, -1]
    assert len(seen) == sum(len(x) for x in m.v_to_v)


def test_reader_errors(tmp_path):
    with pytest.raises(G.GmshError) as e:
        G.GmshMesh(tmp_path / "missing.msh", 2)
    assert e.value.status == 1
    g = GOLDEN["straight_2d_quad_periodic"]["msh"]
    p = tmp_path / "a.msh"
    p.write_text(g.replace("1 1 2 10053 1001 1 5", "1 1 3 10053 1001 7 1 5"))   # three tags
    with pytest.raises(G.GmshError) as e:
        G.GmshMesh(p, 2)
    assert e.value.status == 2
    p.write_text(g.replace("10053 1001", "10077 1001"))                         # an unknown boundary code
    with pytest.raises(G.GmshError) as e:
        G.GmshMesh(p, 2)
    assert e.value.status == 2


def _state(x):
    d = x.shape[1]
    rho = 1.0 + 0.2 * np.sin(0.7 * x[:, 0] + 0.3) * np.cos(0.5 * x[:, 1])
    vel = [0.5 + 0.1 * np.cos(0.4 * x[:, 1]), 0.3 + 0.1 * np.sin(0.6 * x[:, 0])]
    if d == 3:
        vel.append(0.2 + 0.05 * np.sin(0.3 * x[:, 2]))
    p = 1.0 + 0.1 * np.cos(0.3 * x[:, 0] + 0.2 * x[:, 1])
    return np.stack([rho] + [rho * v for v in vel] + [p / P.GM1 + 0.5 * rho * sum(v * v for v in vel)], axis=1)


def _box_problem(tmp_path, d, n, p, seed, flux=P.NUM_FLUX_ROE_PIKE, periodic=True, codes=None):
    path = tmp_path / f"box_{d}_{seed}.msh"
    G.write_box_msh(path, d, n, 0.0, 10.0, periodic=periodic, codes=codes, rotate_seed=seed, perturb=0.2,
                    perturb_seed=3)
    return G.gmsh_tp_problem(path, d, p, P.PDE_EULER, flux, _state, exterior=_state)


@pytest.mark.parametrize("d,n,p,periodic,codes", [
    (2, 4, 3, True, None),
    (3, 3, 2, True, None),
    (2, 4, 2, (True, False), {(1, 0): 10102, (1, 1): 10101}),
    (3, 3, 2, (False, True, False), {(0, 0): 10101, (0, 1): 10101, (2, 0): 10102, (2, 1): 10102})])
def test_rotated_frames_give_the_aligned_residual(tmp_path, d, n, p, periodic, codes):
    pa = _box_problem(tmp_path, d, n, p, None, periodic=periodic, codes=codes)
    pb = _box_problem(tmp_path, d, n, p, 5, periodic=periodic, codes=codes)
    ra, _ = oracle.Oracle(pa).compute_rhs(pa.sol)
    rb, _ = oracle.Oracle(pb).compute_rhs(pb.sol)
    xa, xb = pa.solution_node_xyz(), pb.solution_node_xyz()
    err = 0.0
    for v in range(pa.n_volumes):
        dist = np.linalg.norm(xa[v][:, None, :] - xb[v][None, :, :], axis=2)
        j = np.argmin(dist, axis=1)
        assert dist[np.arange(len(j)), j].max() < 1e-9
        err = max(err, float(np.abs(ra[v] - rb[v][:, j]).max()))
    assert err <= 1e-12 * np.abs(ra).max()
    if d == 3 and periodic is True:
        assert set(pb.mesh.gmsh.face_ord[:, 1]) == set(range(8))   # every QUAD-face ordering occurs


def test_free_stream_on_perturbed_rotated_mesh(tmp_path):
    for d, n in ((2, 4), (3, 3)):
        prob = _box_problem(tmp_path, d, n, 3, 7)
        cs = P.constant_state(prob, [1.0, 0.3, -0.2] + ([0.1] if d == 3 else []) + [2.5])
        assert oracle.Oracle(prob).compute_rhs(cs)[1] < 1e-11


# ---- the reference's curved-boundary workflow: a blended annulus read from a file ----------------------------------
def _couette_fns(omega=1.0):
    def state(x):
        return P.taylor_couette_state(x[:, 0], x[:, 1], 0.5, 1.0, omega, 0.02, 0.72, 1.0, 1.0, 1.0, 0.0).T

    def wall(x):
        r, th = np.hypot(x[:, 0], x[:, 1]), np.arctan2(x[:, 1], x[:, 0])
        e_b = 1.0 / P.GM1 + 0.5 * (omega * 0.5) ** 2
        return np.stack([np.ones_like(r), -np.sin(th) * omega * r, np.cos(th) * omega * r, np.full_like(r, e_b)], 1)
    return state, wall


def _oracle_blend(ve, fc, p):
    from oracle import blend as B
    return np.transpose(B.blend_quad(ve, fc, p), (0, 2, 1))


def test_blended_annulus_from_a_file(tmp_path):
    """gmsh annulus (codes 20113 inside, 20111 outside, random local frames) -> reader -> curved faces from the codes
    -> blend: the same domain as the structured annulus (area), and the fluid at rest is steady on it."""
    from dpgsolver_gb300.host.element import TPOperatorSet
    from dpgsolver_gb300.host.geometry import TPGeometry
    from dpgsolver_gb300.host.mesh import StructuredMesh
    path = tmp_path / "annulus.msh"
    G.write_annulus_msh(path, 3, 16, rotate_seed=4)
    state, wall = _couette_fns(omega=0.0)
    ns = {"viscosity": P.VISCOSITY_CONSTANT, "mu": 0.02, "Pr": 0.72, "r_s": 1.0}
    prob = G.gmsh_tp_problem(path, 2, 3, P.PDE_NAVIER_STOKES, P.NUM_FLUX_ROE_PIKE, state, exterior=wall, ns=ns,
                             blend=_oracle_blend)
    assert sorted(set(prob.bc[prob.mesh.face_vol[:, 1] < 0].tolist())) == [20111, 20113]
    assert int(G.curved_faces(prob.mesh).sum()) == 32
    area = float((prob.geom.jacobian_det_vc * prob.ops.w_vc[None, :]).sum())
    ve, fc = P.annulus_vertices((3, 16))
    mesh = StructuredMesh(2, (3, 16), 0.0, 1.0, periodic=(False, True))
    ops = TPOperatorSet(mesh.e_type, 3)
    ref = TPGeometry(mesh, ops, curved=True, coef=_oracle_blend(ve, fc, 3))
    assert abs(area - float((ref.jacobian_det_vc * ops.w_vc[None, :]).sum())) <= 1e-13
    rest = P.constant_state(prob, [1.0, 0.0, 0.0, 1.0 / P.GM1])
    o = oracle.Oracle(prob)
    assert np.max(np.abs(o.compute_rhs_raw(rest))) < 1e-14
