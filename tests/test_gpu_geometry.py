"""Geometry precompute on the device (dgpu_compute_geometry, dgpu_create with geom_coef) against the host's
restatement of the reference's geometry (dpgsolver_gb300/host/geometry.py, geometry_T.c:165-325).

The two are independent FP64 evaluations of the same interpolation and derivative sums, so they agree to
rounding. The 3D metric terms are a curl of products X_l dX_m/dr of coordinates up to 10 whose entries cancel
down to the element size, so their rounding grows with |X| / h and with p (1.2e-13 at HEX p = 4 on 3^3, 2e-13 on
the 32^3 p = 3 mesh); the bound per array is the residual parity bound, 1e-12 normwise relative. A context built
from the geometry coefficients must give the residual of one built from the host's factors (and the oracle's)
within the same bound.
"""
import ctypes

import numpy as np
import pytest

import oracle
from dpgsolver_gb300 import _lib
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
GEO_TOL = 1e-12
TOL = 1e-12

CASES = {
    "adv2d_straight_p2_6": lambda: P.advection_2d(6, 2),
    "vortex2d_p3_8": lambda: P.euler_vortex_2d(8, 3),
    "vortex2d_p4_4": lambda: P.euler_vortex_2d(4, 4),
    "hex_p1_4": lambda: P.euler_hex_3d(4, 1),
    "hex_p2_4": lambda: P.euler_hex_3d(4, 2),
    "hex_p3_6": lambda: P.euler_hex_3d(6, 3),
    "hex_p4_3": lambda: P.euler_hex_3d(3, 4),
    "duct3d_p3_4": lambda: P.euler_duct_3d(4, 3),
    "channel2d_p3_6": lambda: P.euler_channel_2d(6, 3),
}


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", sorted(CASES))
def test_device_geometry_matches_host(gpu_lib, name):
    from dpgsolver_gb300.solver import compute_geometry
    prob = CASES[name]()
    g = prob.geom
    dev = compute_geometry(prob)
    assert rel(dev["metrics_vc"], g.metrics_vc) <= GEO_TOL
    assert rel(dev["jacobian_det_vc"], g.jacobian_det_vc) <= GEO_TOL
    assert rel(dev["normals_fc"], g.normals_fc) <= GEO_TOL
    assert rel(dev["jacobian_det_fc"], g.jacobian_det_fc) <= GEO_TOL
    assert rel(dev["xyz_fc"], g.xyz_fc) <= GEO_TOL


@pytest.mark.parametrize("name", ["vortex2d_p3_8", "hex_p3_6", "hex_p2_4", "duct3d_p3_4", "adv2d_straight_p2_6"])
def test_context_from_geometry_coefficients(gpu_lib, name):
    from dpgsolver_gb300.solver import Simulation
    prob = CASES[name]()
    r_ref, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    with Simulation(prob) as a, Simulation(prob, device_geometry=True) as b:
        a.compute_rhs()
        b.compute_rhs()
        ra, rb = a.rhs, b.rhs
        a.ssp_rk3_steps(prob.dt, 3)
        b.ssp_rk3_steps(prob.dt, 3)
        sa, sb = a.sol_coef, b.sol_coef
    assert rel(rb, ra) <= TOL
    assert rel(rb, r_ref) <= TOL
    assert rel(sb, sa) <= TOL


def test_device_geometry_preserves_free_stream(gpu_lib):
    """The curl-form metric terms satisfy the discrete metric identities on the curved HEX mesh."""
    from dpgsolver_gb300.solver import Simulation
    for prob in (P.euler_hex_3d(4, 3), P.euler_hex_3d(3, 4), P.euler_vortex_2d(6, 3)):
        vals = [1.0, 0.3, -0.2] + ([0.1] if prob.d == 3 else []) + [2.5]
        with Simulation(prob, device_geometry=True) as sim:
            sim.upload_state(P.constant_state(prob, vals))
            assert sim.compute_rhs() < 1e-11


def test_geometry_errors(gpu_lib):
    from dpgsolver_gb300.solver import Simulation, compute_geometry
    prob = P.euler_hex_3d(3, 2)
    # mirrored coordinates: every Jacobian determinant negative
    prob.geom.X_geom = prob.geom.X_geom * np.array([-1.0, 1.0, 1.0])
    with pytest.raises(_lib.DGPUError) as e:
        compute_geometry(prob)
    assert e.value.status == 1 and "Jacobian" in str(e.value)
    with pytest.raises(_lib.DGPUError) as e:
        Simulation(prob, device_geometry=True)
    assert e.value.status == 1
    prob = P.euler_hex_3d(3, 2)
    prob.geom.p_g = 5
    with pytest.raises(_lib.DGPUError) as e:
        compute_geometry(prob)
    assert e.value.status == 2
    # both the factors and the coefficients: refused
    prob = P.euler_hex_3d(2, 1)
    tp = _lib.TPOperators()
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (prob.ops.cv0_1d, prob.ops.cv1_1d,
                                                                 prob.ops.cv0_bnd_1d, prob.ops.w_vc_1d)]
    tp.elem_type, tp.p = prob.ops.e_type, prob.ops.p
    tp.cv0_vs_vc, tp.cv1_vs_vc, tp.cv0_vs_fc, tp.w_vc = [a.ctypes.data_as(_lib.c_double_p) for a in keep]
    phys = _lib.Physics()
    phys.d, phys.pde, phys.num_flux = 3, prob.pde, prob.num_flux
    g = prob.geom
    arrs = [np.ascontiguousarray(np.transpose(g.metrics_vc, (0, 3, 2, 1))), np.ascontiguousarray(g.jacobian_det_vc),
            np.ascontiguousarray(g.normals_fc), np.ascontiguousarray(g.jacobian_det_fc),
            np.ascontiguousarray(np.transpose(g.X_geom, (0, 2, 1)))]
    fv = np.ascontiguousarray(prob.mesh.face_vol, dtype=np.int32)
    flf = np.ascontiguousarray(prob.mesh.face_lf, dtype=np.int32)
    m = _lib.Mesh()
    m.n_volumes, m.n_faces = prob.n_volumes, prob.mesh.n_faces
    m.face_vol, m.face_lf = fv.ctypes.data_as(_lib.c_int_p), flf.ctypes.data_as(_lib.c_int_p)
    m.metrics_vc, m.jacobian_det_vc, m.normals_fc, m.jacobian_det_fc, m.geom_coef = \
        [a.ctypes.data_as(_lib.c_double_p) for a in arrs]
    m.p_g = 1
    h = ctypes.c_void_p()
    st = gpu_lib.dgpu_create(ctypes.byref(phys), ctypes.byref(tp), ctypes.byref(m), ctypes.byref(h))
    assert st == 1 and b"geom_coef" in gpu_lib.dgpu_last_error(None)


# ---- blended geometry of curved QUAD volumes (dgpu_blend_geometry) ------------------------------------------------
@pytest.mark.parametrize("p_g", [1, 2, 3, 4])
def test_blend_geometry_matches_oracle(gpu_lib, p_g):
    """The device's blend against the oracle's dense-operator restatement (oracle/blend.py) on the annulus, and on
    the same vertices with random curved-face flags (several curved faces per volume, blended one after another)."""
    from oracle import blend as B
    from dpgsolver_gb300.solver import blend_geometry
    for n, seed in (((3, 16), None), ((6, 6), None), ((4, 8), 3)):
        ve, fc = P.annulus_vertices(n, rotate=0.3)
        if seed is not None:
            fc = np.random.default_rng(seed).integers(0, 2, fc.shape).astype(np.int32)
        ref = np.transpose(B.blend_quad(ve, fc, p_g), (0, 2, 1))
        got = blend_geometry(ve, fc, p_g)
        assert np.max(np.abs(got - ref)) <= 1e-14


def test_taylor_couette_on_the_device_blended_geometry(gpu_lib):
    """The reference's Taylor-Couette set-up end to end on the device: straight annulus -> dgpu_blend_geometry ->
    dgpu_create from the geometry coefficients -> residual and RK steps, against the oracle on the same
    coefficients (the host's geometric factors)."""
    from dpgsolver_gb300.solver import Simulation, blend_geometry
    ve, fc = P.annulus_vertices((3, 16))
    coef = blend_geometry(ve, fc, 3)
    prob = P.ns_taylor_couette((3, 16), 3, mu=0.02, perturb=0.2, geom_coef=coef)
    o = oracle.Oracle(prob)
    r_ref, _ = o.compute_rhs(prob.sol)
    floor = 0.0
    for seed in range(3):
        noisy = prob.sol * (1.0 + np.random.default_rng(seed).choice([-1.0, 1.0], prob.sol.shape) * 2.0 ** -52)
        floor = max(floor, rel(o.compute_rhs(noisy)[0], r_ref))
    s_ref = prob.sol.copy()
    for _ in range(3):
        s_ref, _, _ = o.ssp_rk3_step(s_ref, prob.dt)
    with Simulation(prob, device_geometry=True) as sim:
        sim.compute_rhs()
        r = sim.rhs
        sim.ssp_rk3_steps(prob.dt, 3)
        s = sim.sol_coef
    assert rel(r, r_ref) <= max(TOL, 4.0 * floor)
    assert rel(s, s_ref) <= TOL


def test_blend_geometry_refusals(gpu_lib):
    lib = _lib.load()
    ve = np.zeros((1, 2, 4))
    fc = np.zeros((1, 4), dtype=np.int32)
    out = np.zeros((1, 2, 16))
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    args = (ve.ctypes.data_as(dp), fc.ctypes.data_as(ip), out.ctypes.data_as(dp))
    assert lib.dgpu_blend_geometry(3, 3, 1, *args) == 2    # no 3D TP blending in the reference
    assert lib.dgpu_blend_geometry(2, 5, 1, *args) == 2
    assert lib.dgpu_blend_geometry(2, 3, 0, *args) == 1
