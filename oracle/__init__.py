"""ctypes loader for the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle (dg_oracle.c) restates the reference's explicit DG residual with dense operators. Only tests/,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it, always as the checker or the
timed CPU baseline, never as the product.
"""
from __future__ import annotations

import ctypes
import fcntl
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_int_p = ctypes.POINTER(ctypes.c_int)


class _Group(ctypes.Structure):
    _fields_ = [("n_vs", ctypes.c_int), ("n_vc", ctypes.c_int), ("cv0_vs_vc", _c_double_p),
                ("tw1_vt_vc", _c_double_p), ("w_vc", _c_double_p), ("ccSB0", _c_double_p), ("ccBS0", _c_double_p),
                ("cv1_vs_vc", _c_double_p)]


class _FaceOps(ctypes.Structure):
    _fields_ = [("n_fc", ctypes.c_int), ("n_vs", ctypes.c_int), ("cv0_vs_fc", _c_double_p),
                ("tw0_vt_fc", _c_double_p)]


class _Problem(ctypes.Structure):
    _fields_ = [
        ("d", ctypes.c_int), ("n_var", ctypes.c_int), ("pde", ctypes.c_int), ("num_flux", ctypes.c_int),
        ("positivity", ctypes.c_int), ("b_adv", ctypes.c_double * 3),
        ("n_groups", ctypes.c_int), ("groups", ctypes.POINTER(_Group)),
        ("n_face_ops", ctypes.c_int), ("face_ops", ctypes.POINTER(_FaceOps)),
        ("n_volumes", ctypes.c_int), ("vol_group", _c_int_p), ("metrics_vc", _c_double_p),
        ("jacobian_det_vc", _c_double_p),
        ("n_faces", ctypes.c_int), ("face_vol", _c_int_p), ("face_lf", _c_int_p), ("face_ops_idx", _c_int_p),
        ("nc_fc", _c_int_p), ("normals_fc", _c_double_p), ("jacobian_det_fc", _c_double_p),
        ("bc_fc", _c_int_p), ("bc_state_fc", _c_double_p), ("bc_data", ctypes.c_double * 4),
        ("viscosity", ctypes.c_int), ("mu", ctypes.c_double), ("Pr", ctypes.c_double), ("r_s", ctypes.c_double),
        ("dTdn", ctypes.c_double), ("source_vc", _c_double_p),
    ]


def _stale() -> bool:
    return not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("dg_oracle.c", "dg_oracle_T.h", "dg_oracle.h"))


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (processes building at the same time serialise on a lock
    file; the Makefile links to a temporary name and renames, so a loader never sees a partial library)."""
    if force or _stale():
        with open(os.path.join(_HERE, ".build.lock"), "w") as lock:
            fcntl.flock(lock, fcntl.LOCK_EX)
            if force or _stale():
                subprocess.run(["make", "-s", "-B" if force else "-s", "-C", _HERE, "liboracle.so"], check=True)
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
        lib.oracle_face_traces.argtypes = [ctypes.c_void_p, _c_double_p, ctypes.c_int, _c_int_p, _c_double_p]
        lib.oracle_face_traces.restype = ctypes.c_int
        lib.oracle_compute_rhs_remote.argtypes = [ctypes.c_void_p, _c_double_p, _c_double_p, _c_double_p,
                                                  _c_double_p]
        lib.oracle_compute_rhs_remote.restype = ctypes.c_int
        lib.oracle_face_node_total.argtypes = [ctypes.c_void_p]
        lib.oracle_face_node_total.restype = ctypes.c_size_t
        lib.oracle_m_inv.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.oracle_m_inv.restype = _c_double_p
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(_c_double_p)


def _ip(a):
    return a.ctypes.data_as(_c_int_p)


class Oracle:
    """Oracle context for a DG problem (uniform DGProblem or mixed-order MixedTPProblem): dense reference
    operators, the reference's data flow. States are passed in the problem's own shape."""

    def __init__(self, prob):
        from dpgsolver_gb300.host.element import face_operators
        from dpgsolver_gb300.host.problem import flat_arrays

        lib = _load()
        fl = flat_arrays(prob)
        d = prob.d
        keep = []

        def arr(a, dtype=np.float64):
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return a

        groups = fl["groups"]
        G = (_Group * len(groups))()
        for gi, ops in enumerate(groups):
            G[gi].n_vs, G[gi].n_vc = ops.n_vs, ops.n_vc
            G[gi].cv0_vs_vc = _dp(arr(ops.cv0_vs_vc()))
            G[gi].tw1_vt_vc = _dp(arr(np.stack([ops.tw1_vt_vc(k) for k in range(d)])))
            G[gi].w_vc = _dp(arr(ops.w_vc))
            G[gi].ccSB0 = _dp(arr(ops.ccSB0_vs_vs()))      # Bezier maps (enforce_positivity_highorder)
            G[gi].ccBS0 = _dp(arr(ops.ccBS0_vs_vs()))
            if not getattr(ops, "dense", False):
                G[gi].cv1_vs_vc = _dp(arr(np.stack([ops.cv1_vs_vc(k) for k in range(d)])))
        # face operator sets: one per (group, face order, orientation) that occurs, stacked over local faces
        vol_group = fl["vol_group"]
        face_q = fl["face_q"]
        face_ord = fl.get("face_ord")
        mesh = prob.mesh
        pairs = {}
        idx = np.empty((mesh.n_faces, 2), dtype=np.int32)
        for f in range(mesh.n_faces):
            for s in range(2):
                o = int(face_ord[f, s]) if face_ord is not None else 0
                # boundary side / side of another partition: unused, any valid key
                v = mesh.face_vol[f, s] if mesh.face_vol[f, s] >= 0 else mesh.face_vol[f, 1 - s]
                gops = groups[int(vol_group[v])]
                lf_v = mesh.face_lf[f, s] if mesh.face_vol[f, s] >= 0 else mesh.face_lf[f, 1 - s]
                # dense groups: one set per face type too (TRI and QUAD faces have different node counts)
                ft = int(gops.face_type(int(lf_v))) if getattr(gops, "dense", False) else -1
                key = (int(vol_group[v]), int(face_q[f]), o, ft)
                if key not in pairs:
                    pairs[key] = len(pairs)
                idx[f, s] = pairs[key]
        FO = (_FaceOps * len(pairs))()
        for (gi, qf, o, ft), k in pairs.items():
            ops = groups[gi]
            if getattr(ops, "dense", False):
                cv0, tw0 = [], []
                n_fc_ft = None
                for lf in range(ops.n_lf):
                    if ops.face_type(lf) == ft:
                        n_fc_ft = len(ops.w_fc(lf, qf))
                for lf in range(ops.n_lf):
                    if ops.face_type(lf) == ft and o < ops.n_ords(lf):
                        c = ops.cv0_vs_fc(lf, o, qf)
                        t = c.T * ops.w_fc(lf, qf)[None, :]
                    else:   # a local face of the other type, or its orientation: never selected with this set
                        c = np.zeros((n_fc_ft, ops.n_vs))
                        t = c.T.copy()
                    cv0.append(c)
                    tw0.append(t)
            else:
                if o != 0:
                    raise ValueError("TP volumes see their faces unpermuted")
                cv0, tw0, _ = face_operators(ops, qf)
            FO[k].n_fc, FO[k].n_vs = cv0[0].shape[0], ops.n_vs
            FO[k].cv0_vs_fc = _dp(arr(np.stack(cv0)))
            FO[k].tw0_vt_fc = _dp(arr(np.stack(tw0)))

        P = _Problem()
        P.d, P.n_var, P.pde, P.num_flux = d, prob.n_var, prob.pde, prob.num_flux
        P.positivity = 1 if prob.positivity else 0
        for k in range(3):
            P.b_adv[k] = float(prob.b_adv[k])
        P.n_groups, P.groups = len(groups), G
        P.n_face_ops, P.face_ops = len(pairs), FO
        P.n_volumes = mesh.n_volumes
        P.vol_group = _ip(arr(vol_group, np.int32))
        P.metrics_vc = _dp(arr(fl["metrics_vc"]))
        P.jacobian_det_vc = _dp(arr(fl["jacobian_det_vc"]))
        P.n_faces = mesh.n_faces
        P.face_vol = _ip(arr(mesh.face_vol, np.int32))
        P.face_lf = _ip(arr(mesh.face_lf, np.int32))
        P.face_ops_idx = _ip(arr(idx, np.int32))
        P.nc_fc = _ip(arr(fl["nc_fc"], np.int32))
        P.normals_fc = _dp(arr(fl["normals_fc"]))
        P.jacobian_det_fc = _dp(arr(fl["jacobian_det_fc"]))
        if fl.get("bc_fc") is not None:
            n_fc_total = int(sum(FO[idx[f, 0]].n_fc for f in range(mesh.n_faces)))
            if np.size(fl["bc_fc"]) != mesh.n_faces or np.size(fl["bc_state_fc"]) != n_fc_total * prob.n_var:
                raise ValueError("bc_fc needs one code per face and bc_state_fc n_var values per face node")
            P.bc_fc = _ip(arr(fl["bc_fc"], np.int32))
            P.bc_state_fc = _dp(arr(fl["bc_state_fc"]))
            for k, x in enumerate(fl.get("bc_data") or (0.0, 0.0, 0.0, 0.0)):
                P.bc_data[k] = float(x)
        ns = getattr(prob, "ns", None)
        if ns is not None:
            P.viscosity, P.mu, P.Pr, P.r_s = int(ns["viscosity"]), float(ns["mu"]), float(ns["Pr"]), float(ns["r_s"])
            P.dTdn = float(ns.get("dTdn", 0.0))
        if fl.get("source_vc") is not None:
            P.source_vc = _dp(arr(fl["source_vc"]))
        self._keep = (keep, G, FO, P)
        h = ctypes.c_void_p()
        st = lib.oracle_create(ctypes.byref(P), ctypes.byref(h))
        if st != 0:
            raise RuntimeError(f"oracle_create failed: {st}")
        self._h = h
        self._lib = lib
        self.prob = prob
        self.n_state = int(fl["sol"].size)
        self._n_var = int(prob.n_var)
        self._n_fc = int(max(FO[k].n_fc for k in range(len(pairs)))) if len(pairs) else 0

    def __del__(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.oracle_destroy(self._h)
            self._h = None

    def _flat(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != self.n_state:
            raise ValueError(f"state has {a.size} values, the problem {self.n_state}")
        return a.reshape(-1)

    def compute_rhs(self, sol):
        s = self._flat(sol)
        r = np.empty_like(s)
        mx = ctypes.c_double()
        st = self._lib.oracle_compute_rhs(self._h, _dp(s), _dp(r), ctypes.byref(mx))
        if st != 0:
            raise RuntimeError(f"oracle_compute_rhs failed: {st}")
        return r.reshape(np.shape(sol)), mx.value

    def face_traces(self, sol, slots):
        """Traces of the face sides slots (2 f + s), each (n_var, n_fc) in the side's own face-node order."""
        s = self._flat(sol)
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        n_fc = self._n_fc
        out = np.empty((len(sl), self._n_var, n_fc))
        st = self._lib.oracle_face_traces(self._h, _dp(s), len(sl), _ip(sl), _dp(out))
        if st != 0:
            raise RuntimeError(f"oracle_face_traces failed: {st}")
        return out

    def compute_rhs_remote(self, sol, remote):
        """Residual of a partition: remote (n_faces, n_var, n_fc) holds the traces of the faces' sides that belong
        to other partitions (face_vol == -2), in those sides' own face-node order; other entries are ignored."""
        s = self._flat(sol)
        rm = np.ascontiguousarray(remote, dtype=np.float64)
        if rm.size != self._lib.oracle_face_node_total(self._h) * self._n_var:
            raise ValueError("remote traces: one (n_var, n_fc) block per face")
        r = np.empty_like(s)
        mx = ctypes.c_double()
        st = self._lib.oracle_compute_rhs_remote(self._h, _dp(s), _dp(rm), _dp(r), ctypes.byref(mx))
        if st != 0:
            raise RuntimeError(f"oracle_compute_rhs_remote failed: {st}")
        return r.reshape(np.shape(sol)), mx.value

    def compute_rhs_raw(self, sol):
        s = self._flat(sol)
        r = np.empty_like(s)
        st = self._lib.oracle_compute_rhs_raw(self._h, _dp(s), _dp(r))
        if st != 0:
            raise RuntimeError(f"oracle_compute_rhs_raw failed: {st}")
        return r.reshape(np.shape(sol))

    def compute_rhs_cmplx(self, sol_re, sol_im):
        sr = self._flat(sol_re)
        si = self._flat(sol_im)
        rr, ri = np.empty_like(sr), np.empty_like(sr)
        st = self._lib.oracle_compute_rhs_cmplx(self._h, _dp(sr), _dp(si), _dp(rr), _dp(ri))
        if st != 0:
            raise RuntimeError(f"oracle_compute_rhs_cmplx failed: {st}")
        return rr.reshape(np.shape(sol_re)), ri.reshape(np.shape(sol_re))

    def ssp_rk3_step(self, sol, dt):
        """Returns (new_sol, max_rhs, n_corrections) for a copy of sol."""
        s = np.array(self._flat(sol), copy=True)
        mx = ctypes.c_double()
        nc = ctypes.c_int()
        st = self._lib.oracle_ssp_rk3_step(self._h, dt, _dp(s), ctypes.byref(mx), ctypes.byref(nc))
        if st != 0:
            raise RuntimeError(f"oracle_ssp_rk3_step failed: {st}")
        return s.reshape(np.shape(sol)), mx.value, nc.value

    def enforce_positivity(self, sol):
        s = np.array(self._flat(sol), copy=True)
        nc = ctypes.c_int()
        st = self._lib.oracle_enforce_positivity(self._h, _dp(s), ctypes.byref(nc))
        if st != 0:
            raise RuntimeError(f"oracle_enforce_positivity failed: {st}")
        return s.reshape(np.shape(sol)), nc.value

    def m_inv(self, v: int):
        n = self.prob.ops.n_vs if not hasattr(self.prob, "groups") else \
            self.prob.groups[self.prob.vol_group[v]].n_vs
        p = self._lib.oracle_m_inv(self._h, int(v))
        return np.ctypeslib.as_array(p, shape=(n, n)).copy()
