"""The C ABI called from compiled C host code (tests/c/dgpu_caller.c), not through ctypes.

The program keeps the mesh the way the reference does (lists of solver volumes and faces owning their multiarrays),
packs it once in list order, and replaces compute_rhs_dg and time_step_ssp_rk_33 by dgpu_compute_rhs_host and
dgpu_ssp_rk3_step_host. On the CPU it must compile with -Wall -Wextra -Werror against include/dgpu.h and link to
libdgpu.so; on the GPU its residual and RK states must match the reference's own (the golden fixtures of
tests/golden/make_ref_golden.py) to 1e-12: periodic advection and Euler, the duct with total T/p and back-pressure
faces, the supersonic vortex with Riemann faces and slip walls, and the Navier-Stokes Taylor-Couette case with its
walls. The second program (tests/c/dgpu_batch_caller.c) does the same for a p-adapted mesh through the batched
context: the reference's own adapt_hp orders (three per mesh) for advection, the Euler vortex and the Navier-Stokes
Taylor-Couette case.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle
import oracle.reference as R

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "c", "dgpu_caller.c")


BATCH_SRC = os.path.join(REPO, "tests", "c", "dgpu_batch_caller.c")


def build_caller(out_dir, src=SRC):
    import dpgsolver_gb300
    lib = dpgsolver_gb300.build()
    exe = os.path.join(out_dir, os.path.splitext(os.path.basename(src))[0])
    subprocess.run(["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(REPO, "include"),
                    src, "-o", exe, lib, "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def test_c_caller_compiles_against_the_header(tmp_path):
    for src in (SRC, BATCH_SRC):
        assert os.path.exists(build_caller(str(tmp_path), src))


def write_case(path, prob, ref, n_steps):
    """The case in the reference's layouts: per volume metrics_vc (n_vc, d, d) and sol_coef (n_vs, n_var)
    column-major, per face normals_fc (n_fc, d) row-major."""
    ops = prob.ops
    with open(path, "wb") as fh:
        np.array([0x55504744, prob.d, ops.p, prob.pde, prob.num_flux, int(prob.positivity), prob.n_volumes,
                  prob.mesh.n_faces, n_steps], dtype=np.int32).tofile(fh)
        np.array([float(ref["dt"])] + [float(b) for b in prob.b_adv[:3]], dtype=np.float64).tofile(fh)
        ns = getattr(prob, "ns", None) or {}
        np.array([int(ns.get("viscosity", 0))], dtype=np.int32).tofile(fh)
        np.array([ns.get("mu", 0.0), ns.get("Pr", 0.0), ns.get("r_s", 0.0), ns.get("dTdn", 0.0)],
                 dtype=np.float64).tofile(fh)
        np.asarray(prob.bc_data if prob.bc_data is not None else (0.0,) * 4, dtype=np.float64).tofile(fh)
        for a in (ops.cv0_1d, ops.cv1_1d, ops.cv0_bnd_1d, ops.w_vc_1d, ops.ccSB0_1d, ops.ccBS0_1d):
            np.ascontiguousarray(a, dtype=np.float64).tofile(fh)
        met = np.transpose(ref["metrics_vc"], (0, 3, 2, 1))
        for v in range(prob.n_volumes):
            np.ascontiguousarray(met[v]).tofile(fh)
            np.ascontiguousarray(ref["jacobian_det_vc"][v]).tofile(fh)
            np.ascontiguousarray(ref["sol_in"][v]).tofile(fh)
        for f in range(prob.mesh.n_faces):
            bc = int(prob.bc[f]) if prob.bc is not None else 0
            np.concatenate([ref["face_vol"][f], ref["face_lf"][f], ref["face_ord"][f], [bc]]).astype(np.int32).tofile(fh)
            np.ascontiguousarray(ref["normals_fc"][f]).tofile(fh)
            np.ascontiguousarray(ref["jacobian_det_fc"][f]).tofile(fh)
            if ref["face_vol"][f][1] < 0:   # the exterior state at the face nodes, (n_fc, n_var) row-major
                np.ascontiguousarray(prob.bc_state[f]).tofile(fh)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "c2_n8", "c2_lf_n8", "duct_n4", "sduct_n4", "sv_n3", "tc_n2", "tc_diab_n2",
                                  "tc_suth_n2"])
def test_c_caller_matches_reference(gpu_lib, tmp_path, name):
    ref = dict(np.load(os.path.join(REPO, "tests", "golden", f"reference_{name}.npz")))
    prob = R.with_reference_inputs(R.host_problem(name), ref)
    exe = build_caller(str(tmp_path))
    case, out = str(tmp_path / "case.bin"), str(tmp_path / "out.bin")
    n_steps = int(ref["steps"])
    write_case(case, prob, ref, n_steps)
    subprocess.run([exe, case, out], check=True)
    res = np.fromfile(out, dtype=np.float64)
    n = prob.sol.size
    assert res.size == 2 * n + 2
    rhs, mx0, sol, _ = res[:n].reshape(prob.sol.shape), res[n], res[n + 1:2 * n + 1].reshape(prob.sol.shape), res[-1]
    # the residual: max(1e-12, twice its one-ulp noise floor) as the other fixture tests
    o = oracle.Oracle(prob)
    r0, _ = o.compute_rhs(prob.sol)
    noisy = prob.sol * (1.0 + np.random.default_rng(0).choice([-1.0, 1.0], prob.sol.shape) * 2.0 ** -52)
    floor = np.max(np.abs(o.compute_rhs(noisy)[0] - r0)) / np.max(np.abs(r0))
    tol = max(1e-12, 2.0 * floor)
    assert np.max(np.abs(rhs - ref["rhs"])) / np.max(np.abs(ref["rhs"])) <= tol
    assert abs(mx0 - float(ref["max_rhs"])) <= tol * float(ref["max_rhs"])
    assert np.max(np.abs(sol - ref["sol_steps"])) / np.max(np.abs(ref["sol_steps"])) <= 1e-12


def write_mixed_case(path, prob, ref):
    """A p-adapted case in the reference's layouts: one TP operator set per order, per volume its group and its
    blocks at its own order, per face its node count at p_f."""
    d = prob.d
    groups = prob.groups
    with open(path, "wb") as fh:
        np.array([0x48435442, d, prob.pde, prob.num_flux, int(prob.positivity), len(groups), prob.n_volumes,
                  prob.mesh.n_faces, int(ref["steps"])], dtype=np.int32).tofile(fh)
        np.array([float(ref["dt"])] + [float(b) for b in prob.b_adv[:3]], dtype=np.float64).tofile(fh)
        ns = getattr(prob, "ns", None) or {}
        np.array([int(ns.get("viscosity", 0))], dtype=np.int32).tofile(fh)
        np.array([ns.get("mu", 0.0), ns.get("Pr", 0.0), ns.get("r_s", 0.0), ns.get("dTdn", 0.0)],
                 dtype=np.float64).tofile(fh)
        np.asarray(prob.bc_data if prob.bc_data is not None else (0.0,) * 4, dtype=np.float64).tofile(fh)
        source = getattr(prob, "source_vc", None)
        np.array([0 if source is None else 1], dtype=np.int32).tofile(fh)
        for ops in groups:
            np.array([ops.p], dtype=np.int32).tofile(fh)
            for a in (ops.cv0_1d, ops.cv1_1d, ops.cv0_bnd_1d, ops.w_vc_1d, ops.ccSB0_1d, ops.ccBS0_1d):
                np.ascontiguousarray(a, dtype=np.float64).tofile(fh)
        nv = prob.n_var
        n_vc = np.array([groups[g].n_vc for g in prob.vol_group], dtype=np.int64)
        vc_off = np.concatenate([[0], np.cumsum(n_vc)])
        for v in range(prob.n_volumes):
            np.array([prob.vol_group[v]], dtype=np.int32).tofile(fh)
            a, b = vc_off[v], vc_off[v + 1]
            np.ascontiguousarray(ref["metrics_vc"][a * d * d:b * d * d]).tofile(fh)
            np.ascontiguousarray(ref["jacobian_det_vc"][a:b]).tofile(fh)
            np.ascontiguousarray(ref["sol_in"][a * nv:b * nv]).tofile(fh)
            if source is not None:   # the same (n_vc, n_var) column-major block layout as sol_coef
                np.ascontiguousarray(np.asarray(source).ravel()[a * nv:b * nv]).tofile(fh)
        fo = prob.face_off
        for f in range(prob.mesh.n_faces):
            bc = int(prob.bc[f]) if prob.bc is not None else 0
            nfc = int(fo[f + 1] - fo[f])
            np.concatenate([ref["face_vol"][f], ref["face_lf"][f], [bc, nfc]]).astype(np.int32).tofile(fh)
            np.ascontiguousarray(ref["normals_fc"][fo[f] * d:fo[f + 1] * d]).tofile(fh)
            np.ascontiguousarray(ref["jacobian_det_fc"][fo[f]:fo[f + 1]]).tofile(fh)
            if ref["face_vol"][f][1] < 0:
                np.ascontiguousarray(prob.bc_state[fo[f]:fo[f + 1]]).tofile(fh)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(R.MIXED_CASES))
def test_c_batch_caller_matches_reference(gpu_lib, tmp_path, name):
    ref = dict(np.load(os.path.join(REPO, "tests", "golden", f"reference_{name}.npz")))
    prob = R.with_reference_mixed_inputs(R.host_mixed_problem(name, ref["p_vol"], ref["face_vol"], ref["face_lf"]),
                                         ref)
    exe = build_caller(str(tmp_path), BATCH_SRC)
    case, out = str(tmp_path / "case.bin"), str(tmp_path / "out.bin")
    write_mixed_case(case, prob, ref)
    subprocess.run([exe, case, out], check=True)
    res = np.fromfile(out, dtype=np.float64)
    n = prob.sol.size
    assert res.size == 2 * n + 2
    rhs, mx0, sol = res[:n], res[n], res[n + 1:2 * n + 1]
    o = oracle.Oracle(prob)
    r0, _ = o.compute_rhs(prob.sol)
    noisy = prob.sol * (1.0 + np.random.default_rng(0).choice([-1.0, 1.0], prob.sol.shape) * 2.0 ** -52)
    floor = np.max(np.abs(o.compute_rhs(noisy)[0] - r0)) / np.max(np.abs(r0))
    # as tests/test_gpu_reference.py: 4 x the floor for the cases of R.WIDE_FLOOR, 2 x elsewhere
    tol = max(1e-12, (4.0 if name in R.WIDE_FLOOR else 2.0) * floor)
    assert np.max(np.abs(rhs - ref["rhs"])) / np.max(np.abs(ref["rhs"])) <= tol
    assert abs(mx0 - float(ref["max_rhs"])) <= tol * float(ref["max_rhs"])
    assert np.max(np.abs(sol - ref["sol_steps"])) / np.max(np.abs(ref["sol_steps"])) <= 1e-12
