"""dgpu_compute_rhs_noalloc: the residual for callers that cannot allocate device memory.

Such a caller (an application whose GPU memory belongs to its own pool, or a loop that must not allocate while it
runs) owns every buffer and hands the library device pointers; the library keeps its intermediates in one fixed
array of its own instead of calling cudaMalloc. Here torch plays that caller: it owns the device buffers. The
result must equal the context entry point's (dgpu_compute_rhs) within the parity tolerance of the other GPU tests,
on two calls in a row (the second call reuses the array the first one left behind).
"""
import ctypes

import numpy as np
import pytest

from dpgsolver_gb300 import _lib
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12  # normwise relative, as in test_gpu_parity.py


def _device_inputs(prob):
    """Caller-owned device copies of the state and of the mesh arrays, in dgpu_create's layouts."""
    import torch
    dev = torch.device("cuda", 0)
    g = prob.geom

    def t(a, dtype=torch.float64):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dtype=dtype, device=dev)

    bufs = {
        "sol": t(prob.sol),
        "rhs": torch.full(prob.sol.shape, float("nan"), dtype=torch.float64, device=dev),
        "met": t(np.transpose(g.metrics_vc, (0, 3, 2, 1))),
        "jac": t(g.jacobian_det_vc),
        "fv": t(prob.mesh.face_vol.astype(np.int32), torch.int32),
        "flf": t(prob.mesh.face_lf.astype(np.int32), torch.int32),
        "nc": t(prob.nc_fc().astype(np.int32), torch.int32),
        "nrm": t(g.normals_fc),
        "jf": t(g.jacobian_det_fc),
    }
    return bufs


def _host_structs(prob, bufs):
    ops = prob.ops
    keep = []

    def hp(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return a.ctypes.data_as(_lib.c_double_p)

    phys = _lib.Physics()
    phys.d, phys.pde, phys.num_flux, phys.positivity = prob.d, prob.pde, prob.num_flux, 0
    for k in range(3):
        phys.b_adv[k] = float(prob.b_adv[k])
    tp = _lib.TPOperators()
    tp.elem_type, tp.p = ops.e_type, ops.p
    tp.cv0_vs_vc, tp.cv1_vs_vc = hp(ops.cv0_1d), hp(ops.cv1_1d)
    tp.cv0_vs_fc, tp.w_vc = hp(ops.cv0_bnd_1d), hp(ops.w_vc_1d)
    tp.ccSB0_vs_vs, tp.ccBS0_vs_vs = hp(ops.ccSB0_1d), hp(ops.ccBS0_1d)

    def dp(name):
        return ctypes.cast(bufs[name].data_ptr(), _lib.c_double_p)

    def ip(name):
        return ctypes.cast(bufs[name].data_ptr(), _lib.c_int_p)

    m = _lib.Mesh()
    m.n_volumes, m.n_faces = prob.mesh.n_volumes, prob.mesh.n_faces
    m.metrics_vc, m.jacobian_det_vc = dp("met"), dp("jac")
    m.face_vol, m.face_lf, m.nc_fc = ip("fv"), ip("flf"), ip("nc")
    m.normals_fc, m.jacobian_det_fc = dp("nrm"), dp("jf")
    return phys, tp, m, keep


def _noalloc_rhs(lib, prob, bufs, structs):
    import torch
    phys, tp, m, _ = structs
    mx = ctypes.c_double()
    st = lib.dgpu_compute_rhs_noalloc(ctypes.byref(phys), ctypes.byref(tp), ctypes.byref(m),
                                      ctypes.c_void_p(bufs["sol"].data_ptr()), ctypes.c_void_p(bufs["rhs"].data_ptr()),
                                      ctypes.byref(mx), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, None)
    return bufs["rhs"].cpu().numpy().copy(), mx.value


@pytest.mark.parametrize("mk", [lambda: P.euler_hex_3d(6, 3), lambda: P.euler_vortex_2d(12, 3),
                                lambda: P.advection_2d(16, 2)])
def test_noalloc_matches_context_entry_twice(gpu_lib, mk):
    from dpgsolver_gb300.solver import Simulation
    prob = mk()
    with Simulation(prob) as sim:
        mx_ref = sim.compute_rhs()
        r_ref = sim.rhs
    bufs = _device_inputs(prob)
    structs = _host_structs(prob, bufs)
    for _ in range(2):
        bufs["rhs"].fill_(float("nan"))
        r, mx = _noalloc_rhs(gpu_lib, prob, bufs, structs)
        assert np.max(np.abs(r - r_ref)) / np.max(np.abs(r_ref)) <= TOL
        assert abs(mx - mx_ref) <= TOL * mx_ref


def test_noalloc_after_other_mesh_and_oversize_rejected(gpu_lib):
    """A smaller mesh after a larger one (stale contents in the shared array) still matches, and a mesh beyond
    the fixed array is refused with an error, not run."""
    from dpgsolver_gb300.solver import Simulation
    big = P.euler_hex_3d(20, 3)          # about 8,000 elements: more than the fixed array holds
    bufs = _device_inputs(big)
    structs = _host_structs(big, bufs)
    phys, tp, m, _ = structs
    st = gpu_lib.dgpu_compute_rhs_noalloc(ctypes.byref(phys), ctypes.byref(tp), ctypes.byref(m),
                                          ctypes.c_void_p(bufs["sol"].data_ptr()),
                                          ctypes.c_void_p(bufs["rhs"].data_ptr()), None, None)
    assert st == 1
    assert b"bytes of scratch" in gpu_lib.dgpu_last_error(None)
    del bufs, structs
    for prob in (P.euler_hex_3d(8, 2), P.euler_hex_3d(4, 2)):
        with Simulation(prob) as sim:
            sim.compute_rhs()
            r_ref = sim.rhs
        b = _device_inputs(prob)
        s = _host_structs(prob, b)
        r, _ = _noalloc_rhs(gpu_lib, prob, b, s)
        assert np.max(np.abs(r - r_ref)) / np.max(np.abs(r_ref)) <= TOL


def test_noalloc_rejects_bad_inputs_without_running(gpu_lib):
    """A face list that gives one (volume, local face) to two face sides, and a state in page-locked host memory
    instead of device memory, are refused with DGPU_ERR_INVALID_ARGUMENT and the residual is left untouched."""
    import torch
    from dpgsolver_gb300.solver import Simulation
    prob = P.euler_hex_3d(4, 2)
    bufs = _device_inputs(prob)
    structs = _host_structs(prob, bufs)
    phys, tp, m, _ = structs

    # one face more than the mesh has, repeating face 0: every (volume, local face) is still covered, face 0's twice
    dup = {k: torch.cat([bufs[k], bufs[k][:1]]) for k in ("fv", "flf", "nc", "nrm", "jf")}
    m_dup = _lib.Mesh()
    m_dup.n_volumes, m_dup.n_faces = m.n_volumes, m.n_faces + 1
    m_dup.metrics_vc, m_dup.jacobian_det_vc = m.metrics_vc, m.jacobian_det_vc
    m_dup.face_vol = ctypes.cast(dup["fv"].data_ptr(), _lib.c_int_p)
    m_dup.face_lf = ctypes.cast(dup["flf"].data_ptr(), _lib.c_int_p)
    m_dup.nc_fc = ctypes.cast(dup["nc"].data_ptr(), _lib.c_int_p)
    m_dup.normals_fc = ctypes.cast(dup["nrm"].data_ptr(), _lib.c_double_p)
    m_dup.jacobian_det_fc = ctypes.cast(dup["jf"].data_ptr(), _lib.c_double_p)
    bufs["rhs"].fill_(float("nan"))
    st = gpu_lib.dgpu_compute_rhs_noalloc(ctypes.byref(phys), ctypes.byref(tp), ctypes.byref(m_dup),
                                          ctypes.c_void_p(bufs["sol"].data_ptr()),
                                          ctypes.c_void_p(bufs["rhs"].data_ptr()), None, None)
    assert st == 1 and b"bad mesh" in gpu_lib.dgpu_last_error(None)
    assert torch.isnan(bufs["rhs"]).all()

    pinned = bufs["sol"].cpu().pin_memory()
    st = gpu_lib.dgpu_compute_rhs_noalloc(ctypes.byref(phys), ctypes.byref(tp), ctypes.byref(m),
                                          ctypes.c_void_p(pinned.data_ptr()),
                                          ctypes.c_void_p(bufs["rhs"].data_ptr()), None, None)
    assert st == 1 and b"device memory of the current device" in gpu_lib.dgpu_last_error(None)
    assert torch.isnan(bufs["rhs"]).all()

    # the same arrays, well formed, still work afterwards
    with Simulation(prob) as sim:
        sim.compute_rhs()
        r_ref = sim.rhs
    r, _ = _noalloc_rhs(gpu_lib, prob, bufs, structs)
    assert np.max(np.abs(r - r_ref)) / np.max(np.abs(r_ref)) <= TOL
