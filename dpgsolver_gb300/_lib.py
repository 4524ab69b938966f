"""Build and load libdgpu.so (the sm_103a CUDA library behind include/dgpu.h) through ctypes.

The library is compiled in-tree with nvcc for sm_103a only. There is no fallback: if the library is missing
or no GB300 is present, every call raises.
"""
from __future__ import annotations

import ctypes
import fcntl
import os
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
LIB_PATH = os.path.join(PKG_DIR, "libdgpu.so")
SOURCES = ["dgpu.cu", "dgpu_batched.cu", "dgpu_mesh_io.cpp"]
HEADERS = ["dgpu_ns.cuh", "dgpu_geometry.cuh", "dgpu_jacobian.cuh", "dgpu_tp.cuh", "dgpu_physics.cuh", "dgpu_dual.cuh", "dgpu_adjoint.cuh", "dgpu_batched.cuh",
           "dgpu_dense.cuh", "dgpu_jvp.cuh", "dgpu_host_ops.h"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo",
              "-Xcompiler", "-fPIC"]
BUILD_DIR = os.path.join(PKG_DIR, "_build")


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(REPO_DIR, "include", h)
                                                                           for h in ("dgpu.h", "dgpu_mesh.h")]
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libdgpu.so for sm_103a (nvcc cross-compiles without a GPU). Processes that build at the same time
    (a test run and a benchmark started together) serialise on a lock file; the later one finds the library fresh."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    with open(os.path.join(BUILD_DIR, "build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not force and not _stale():
            return LIB_PATH
        return _build_locked(verbose)


def _build_locked(verbose: bool) -> str:
    objs, procs = [], []
    for src in SOURCES:   # translation units compile in parallel, then one link
        obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc_path()] + NVCC_FLAGS + ["-c", "-o", obj, os.path.join(CSRC, src)]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd)))
        objs.append(obj)
    for cmd, pr in procs:
        if pr.wait() != 0:
            raise subprocess.CalledProcessError(pr.returncode, cmd)
    tmp = f"{LIB_PATH}.{os.getpid()}.tmp"
    subprocess.run([nvcc_path(), "-shared", "-o", tmp] + objs, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)


class Physics(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("pde", ctypes.c_int), ("num_flux", ctypes.c_int),
                ("positivity", ctypes.c_int), ("b_adv", ctypes.c_double * 3), ("viscosity", ctypes.c_int),
                ("mu", ctypes.c_double), ("Pr", ctypes.c_double), ("r_s", ctypes.c_double),
                ("dTdn", ctypes.c_double)]


class TPOperators(ctypes.Structure):
    _fields_ = [("elem_type", ctypes.c_int), ("p", ctypes.c_int),
                ("cv0_vs_vc", c_double_p), ("cv1_vs_vc", c_double_p), ("cv0_vs_fc", c_double_p),
                ("w_vc", c_double_p), ("ccSB0_vs_vs", c_double_p), ("ccBS0_vs_vs", c_double_p)]


class DenseOperators(ctypes.Structure):
    _fields_ = [("elem_type", ctypes.c_int), ("p", ctypes.c_int), ("n_vs", ctypes.c_int), ("n_vc", ctypes.c_int),
                ("cv0_vs_vc", c_double_p), ("cv1_vs_vc", c_double_p), ("w_vc", c_double_p),
                ("n_lf", ctypes.c_int), ("n_ord", ctypes.c_int), ("n_fc", c_int_p),
                ("cv0_vs_fc", ctypes.POINTER(c_double_p)), ("w_fc", ctypes.POINTER(c_double_p)),
                ("n_tri_vs", ctypes.c_int), ("n_tri_vc", ctypes.c_int), ("n_line_vs", ctypes.c_int),
                ("n_line_vc", ctypes.c_int), ("tri_cv0", c_double_p), ("tri_cv1", c_double_p),
                ("line_cv0", c_double_p), ("line_cv1", c_double_p),
                ("ccSB0_vs_vs", c_double_p), ("ccBS0_vs_vs", c_double_p)]


class Group(ctypes.Structure):
    _fields_ = [("tp", ctypes.POINTER(TPOperators)), ("dense", ctypes.POINTER(DenseOperators))]


class GmshSizes(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("d", "n_nodes", "n_elements", "n_node_nums", "n_periodic", "n_volumes",
                                             "n_volume_faces", "n_ve_bc", "n_faces", "has_periodic")]


class Mesh(ctypes.Structure):
    _fields_ = [("n_volumes", ctypes.c_int), ("metrics_vc", c_double_p), ("jacobian_det_vc", c_double_p),
                ("n_faces", ctypes.c_int), ("face_vol", c_int_p), ("face_lf", c_int_p), ("nc_fc", c_int_p),
                ("normals_fc", c_double_p), ("jacobian_det_fc", c_double_p), ("bc_fc", c_int_p),
                ("bc_state_fc", c_double_p), ("bc_data", c_double_p), ("p_g", ctypes.c_int),
                ("geom_coef", c_double_p)]


EXPORTS = {
    # name: (restype, argtypes)
    "dgpu_create": (ctypes.c_int, [ctypes.POINTER(Physics), ctypes.POINTER(TPOperators), ctypes.POINTER(Mesh),
                                   ctypes.POINTER(ctypes.c_void_p)]),
    "dgpu_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dgpu_gmsh_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "dgpu_gmsh_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dgpu_gmsh_last_error": (ctypes.c_char_p, []),
    "dgpu_gmsh_get_sizes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(GmshSizes)]),
    "dgpu_gmsh_data": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p,
                                      c_int_p]),
    "dgpu_gmsh_connectivity": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    "dgpu_gmsh_vertices": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    "dgpu_gmsh_faces": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    "dgpu_jacobian_structure": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                               ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int)]),
    "dgpu_jacobian_bsr": (ctypes.c_int, [ctypes.c_void_p, c_double_p, ctypes.c_int, c_int_p, c_int_p,
                                         ctypes.c_void_p]),
    "dgpu_compute_geometry": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(TPOperators), ctypes.POINTER(Mesh),
                                             c_double_p, c_double_p, c_double_p, c_double_p, c_double_p]),
    "dgpu_state_size": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "dgpu_upload_state": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_download_state": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_download_rhs": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_compute_rhs": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_compute_rhs_host": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p, c_double_p]),
    "dgpu_ssp_rk3_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, c_double_p]),
    "dgpu_ssp_rk3_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, c_double_p]),
    "dgpu_ssp_rk3_step_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, c_double_p, c_double_p, c_double_p]),
    "dgpu_positivity_corrections": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "dgpu_kernel_launches": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "dgpu_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "dgpu_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dgpu_set_source": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_halo_setup": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_int_p, c_int_p]),
    "dgpu_halo_buffers": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                         ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_size_t)]),
    "dgpu_get_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "dgpu_halo_rhs_begin": (ctypes.c_int, [ctypes.c_void_p]),
    "dgpu_halo_rhs_end": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_halo_stage_begin": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dgpu_halo_stage_end": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, c_double_p]),
    "dgpu_set_kernel_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dgpu_kernel_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, c_double_p,
                                        ctypes.POINTER(ctypes.c_longlong)]),
    "dgpu_probe_fp64": (ctypes.c_int, [ctypes.c_int, c_double_p]),
    "dgpu_probe_fp64_mma": (ctypes.c_int, [ctypes.c_int, c_double_p]),
    "dgpu_blend_geometry": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_int_p, c_double_p]),
    "dgpu_vjp_forward": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p, c_double_p]),
    "dgpu_jvp": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p, c_double_p, c_double_p]),
    "dgpu_vjp_backward": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p]),
    "dgpu_set_objective_faces": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_int_p]),
    "dgpu_objective": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p, c_double_p]),
    "dgpu_adjoint_ssp_rk3": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_size_t,
                                            c_double_p, c_double_p, c_double_p, c_int_p]),
    "dgpu_compute_rhs_noalloc": (ctypes.c_int, [ctypes.POINTER(Physics), ctypes.POINTER(TPOperators),
                                                ctypes.POINTER(Mesh), ctypes.c_void_p, ctypes.c_void_p, c_double_p,
                                                ctypes.c_void_p]),
    "dgpu_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "dgpu_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    # batched mixed-order context
    "dgpu_batch_create": (ctypes.c_int, [ctypes.POINTER(Physics), ctypes.c_int, ctypes.POINTER(TPOperators), c_int_p,
                                         ctypes.POINTER(Mesh), ctypes.POINTER(ctypes.c_void_p)]),
    "dgpu_batch_create_groups": (ctypes.c_int, [ctypes.POINTER(Physics), ctypes.c_int, ctypes.POINTER(Group), c_int_p,
                                                ctypes.POINTER(Mesh), c_int_p, ctypes.POINTER(ctypes.c_void_p)]),
    "dgpu_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dgpu_batch_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "dgpu_batch_state_size": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "dgpu_batch_upload_state": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_batch_set_source": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_batch_set_barrier_timeout": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "dgpu_batch_download_state": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_batch_download_rhs": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_batch_compute_rhs": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dgpu_batch_ssp_rk3_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, c_double_p]),
    "dgpu_batch_set_mode": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dgpu_batch_get_mode": (ctypes.c_int, [ctypes.c_void_p, c_int_p]),
    "dgpu_batch_set_graphs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dgpu_batch_set_group_tile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "dgpu_batch_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_char_p,
                                           ctypes.c_size_t]),
    "dgpu_batch_kernel_launches": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "dgpu_batch_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dgpu_batch_positivity_corrections": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
}


def load(build_if_missing: bool = True):
    """Load libdgpu.so; raises if it cannot be built or loaded (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is missing: call dpgsolver_gb300.build()")
        build()
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class DGPUError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"dgpu status {status}: {message}")
        self.status = status


def check(status: int, ctx=None, batch: bool = False):
    if status != 0:
        lib = load()
        msg = lib.dgpu_batch_last_error(ctx) if batch else lib.dgpu_last_error(ctx)
        raise DGPUError(status, (msg or b"").decode() or lib.dgpu_status_string(status).decode())
