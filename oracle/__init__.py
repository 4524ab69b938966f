"""ctypes loader for the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle (dg_oracle.c) restates the reference's explicit DG residual with dense operators. Only tests/,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it, always as the checker or the
timed CPU baseline, never as the product.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_int_p = ctypes.POINTER(ctypes.c_int)


class _Problem(ctypes.Structure):
    _fields_ = [
        ("d", ctypes.c_int), ("n_var", ctypes.c_int), ("pde", ctypes.c_int), ("num_flux", ctypes.c_int),
        ("positivity", ctypes.c_int), ("b_adv", ctypes.c_double * 3),
        ("n_vs", ctypes.c_int), ("n_vc", ctypes.c_int), ("n_fc", ctypes.c_int),
        ("cv0_vs_vc", _c_double_p), ("tw1_vt_vc", _c_double_p), ("cv0_vs_fc", _c_double_p),
        ("tw0_vt_fc", _c_double_p), ("w_vc", _c_double_p), ("ccSB0", _c_double_p), ("ccBS0", _c_double_p),
        ("n_volumes", ctypes.c_int), ("metrics_vc", _c_double_p), ("jacobian_det_vc", _c_double_p),
        ("n_faces", ctypes.c_int), ("face_vol", _c_int_p), ("face_lf", _c_int_p), ("nc_fc", _c_int_p),
        ("normals_fc", _c_double_p), ("jacobian_det_fc", _c_double_p),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(os.path.join(_HERE, f))
                                               for f in ("dg_oracle.c", "dg_oracle_T.h", "dg_oracle.h")):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(_LIB_PATH)
        lib.oracle_create.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(ctypes.c_void_p)]
        lib.oracle_create.restype = ctypes.c_int
        lib.oracle_destroy.argtypes = [ctypes.c_void_p]
        lib.oracle_destroy.restype = None
        lib.oracle_compute_rhs.argtypes = [ctypes.c_void_p, _c_double_p, _c_double_p, _c_double_p]
        lib.oracle_compute_rhs.restype = ctypes.c_int
        lib.oracle_compute_rhs_raw.argtypes = [ctypes.c_void_p, _c_double_p, _c_double_p]
        lib.oracle_compute_rhs_raw.restype = ctypes.c_int
        lib.oracle_compute_rhs_cmplx.argtypes = [ctypes.c_void_p, _c_double_p, _c_double_p, _c_double_p,
                                                 _c_double_p]
        lib.oracle_compute_rhs_cmplx.restype = ctypes.c_int
        lib.oracle_ssp_rk3_step.argtypes = [ctypes.c_void_p, ctypes.c_double, _c_double_p, _c_double_p,
                                            _c_int_p]
        lib.oracle_ssp_rk3_step.restype = ctypes.c_int
        lib.oracle_enforce_positivity.argtypes = [ctypes.c_void_p, _c_double_p, _c_int_p]
        lib.oracle_enforce_positivity.restype = ctypes.c_int
        lib.oracle_m_inv.argtypes = [ctypes.c_void_p]
        lib.oracle_m_inv.restype = _c_double_p
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(_c_double_p)


def _ip(a):
    return a.ctypes.data_as(_c_int_p)


class Oracle:
    """Oracle context for one DGProblem (dense reference operators, reference data flow)."""

    def __init__(self, prob):
        lib = _load()
        ops, mesh, geom = prob.ops, prob.mesh, prob.geom
        d = prob.d
        keep = {}

        def arr(name, a, dtype=np.float64):
            keep[name] = np.ascontiguousarray(a, dtype=dtype)
            return keep[name]

        P = _Problem()
        P.d, P.n_var, P.pde, P.num_flux = d, prob.n_var, prob.pde, prob.num_flux
        P.positivity = 1 if prob.positivity else 0
        for k in range(3):
            P.b_adv[k] = float(prob.b_adv[k])
        P.n_vs, P.n_vc, P.n_fc = ops.n_vs, ops.n_vc, ops.n_fc
        P.cv0_vs_vc = _dp(arr("cv0", ops.cv0_vs_vc()))
        P.tw1_vt_vc = _dp(arr("tw1", np.stack([ops.tw1_vt_vc(k) for k in range(d)])))
        P.cv0_vs_fc = _dp(arr("cv0f", np.stack([ops.cv0_vs_fc(lf) for lf in range(2 * d)])))
        P.tw0_vt_fc = _dp(arr("tw0f", np.stack([ops.tw0_vt_fc(lf) for lf in range(2 * d)])))
        P.w_vc = _dp(arr("w", ops.w_vc))
        P.ccSB0 = _dp(arr("sb", ops.ccSB0_vs_vs()))
        P.ccBS0 = _dp(arr("bs", ops.ccBS0_vs_vs()))
        P.n_volumes = mesh.n_volumes
        # metrics (nv, n_vc, d, d) -> per volume column-major (n, i, j): index n + n_vc*(i + d*j)
        P.metrics_vc = _dp(arr("m", np.transpose(geom.metrics_vc, (0, 3, 2, 1))))
        P.jacobian_det_vc = _dp(arr("J", geom.jacobian_det_vc))
        P.n_faces = mesh.n_faces
        P.face_vol = _ip(arr("fv", mesh.face_vol, np.int32))
        P.face_lf = _ip(arr("flf", mesh.face_lf, np.int32))
        P.nc_fc = _ip(arr("nc", prob.nc_fc(), np.int32))
        P.normals_fc = _dp(arr("nrm", geom.normals_fc))
        P.jacobian_det_fc = _dp(arr("Jf", geom.jacobian_det_fc))
        h = ctypes.c_void_p()
        st = lib.oracle_create(ctypes.byref(P), ctypes.byref(h))
        if st != 0:
            raise RuntimeError(f"oracle_create failed: {st}")
        self._h = h
        self._lib = lib
        self.prob = prob
        self.shape = prob.sol.shape

    def __del__(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.oracle_destroy(self._h)
            self._h = None

    def compute_rhs(self, sol):
        s = np.ascontiguousarray(sol, dtype=np.float64)
        r = np.empty_like(s)
        mx = ctypes.c_double()
        st = self._lib.oracle_compute_rhs(self._h, _dp(s), _dp(r), ctypes.byref(mx))
        if st != 0:
            raise RuntimeError(f"oracle_compute_rhs failed: {st}")
        return r, mx.value

    def compute_rhs_raw(self, sol):
        s = np.ascontiguousarray(sol, dtype=np.float64)
        r = np.empty_like(s)
        st = self._lib.oracle_compute_rhs_raw(self._h, _dp(s), _dp(r))
        if st != 0:
            raise RuntimeError(f"oracle_compute_rhs_raw failed: {st}")
        return r

    def compute_rhs_cmplx(self, sol_re, sol_im):
        sr = np.ascontiguousarray(sol_re, dtype=np.float64)
        si = np.ascontiguousarray(sol_im, dtype=np.float64)
        rr, ri = np.empty_like(sr), np.empty_like(sr)
        st = self._lib.oracle_compute_rhs_cmplx(self._h, _dp(sr), _dp(si), _dp(rr), _dp(ri))
        if st != 0:
            raise RuntimeError(f"oracle_compute_rhs_cmplx failed: {st}")
        return rr, ri

    def ssp_rk3_step(self, sol, dt):
        """In-place on a copy; returns (new_sol, max_rhs, n_corrections)."""
        s = np.array(sol, dtype=np.float64, copy=True, order="C")
        mx = ctypes.c_double()
        nc = ctypes.c_int()
        st = self._lib.oracle_ssp_rk3_step(self._h, dt, _dp(s), ctypes.byref(mx), ctypes.byref(nc))
        if st != 0:
            raise RuntimeError(f"oracle_ssp_rk3_step failed: {st}")
        return s, mx.value, nc.value

    def enforce_positivity(self, sol):
        s = np.array(sol, dtype=np.float64, copy=True, order="C")
        nc = ctypes.c_int()
        st = self._lib.oracle_enforce_positivity(self._h, _dp(s), ctypes.byref(nc))
        if st != 0:
            raise RuntimeError(f"oracle_enforce_positivity failed: {st}")
        return s, nc.value

    def m_inv(self):
        n = self.prob.ops.n_vs
        p = self._lib.oracle_m_inv(self._h)
        return np.ctypeslib.as_array(p, shape=(self.prob.n_volumes, n, n)).copy()
