"""Host-side mirror of the reference's explicit DG entry points, over the C ABI of include/dgpu.h.

    sim = Simulation(problem)             # constructor_derived_computational_elements + m_inv set-up
    max_rhs = compute_rhs_dg(sim)         # solvers/dg/solve_dg.c:130-136
    max_rhs = time_step_ssp_rk_33(dt, sim)  # solvers/solve_explicit.c:252-301 (static there)
    solve_explicit(sim, n_steps)          # the time loop of solvers/solve_explicit.c:78-118

``sim.sol_coef`` / ``sim.rhs`` give the per-volume (n_vs x n_var) column-major blocks, as arrays of shape
(n_volumes, n_var, n_vs). Errors raise DGPUError with the library's status; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import DGPUError, check  # noqa: F401  (re-exported)


def _dp(a):
    return a.ctypes.data_as(_lib.c_double_p)


def _ip(a):
    return a.ctypes.data_as(_lib.c_int_p)


def _geom_coef(prob):
    """Solver_Volume_T::geom_coef of every volume, (n_volumes, d, n_g): per volume the (n_g x d) column-major
    block of the coordinates at the GLL geometry nodes."""
    return np.ascontiguousarray(np.transpose(prob.geom.X_geom, (0, 2, 1)))


def blend_geometry(xyz_ve, face_curved, p_g: int):
    """Blended geometry coefficients of curved QUAD volumes computed on the device (dgpu_blend_geometry): xyz_ve
    (n_volumes, 2, 4) straight vertices, face_curved (n_volumes, 4) -> (n_volumes, (p_g+1)^2, 2), the coordinates at
    the GLL nodes of order p_g (the layout of TPGeometry's coef)."""
    lib = _lib.load()
    ve = np.ascontiguousarray(xyz_ve, dtype=np.float64)
    fc = np.ascontiguousarray(face_curved, dtype=np.int32)
    nv, n_g = ve.shape[0], (p_g + 1) ** 2
    if ve.shape != (nv, 2, 4) or fc.shape != (nv, 4):
        raise ValueError("xyz_ve must be (n_volumes, 2, 4) and face_curved (n_volumes, 4)")
    out = np.empty((nv, 2, n_g))
    check(lib.dgpu_blend_geometry(2, p_g, nv, _dp(ve), _ip(fc), _dp(out)), None)
    return np.ascontiguousarray(np.transpose(out, (0, 2, 1)))


def compute_geometry(prob):
    """The geometric factors of a TP DGProblem computed on the device from its geometry coefficients
    (dgpu_compute_geometry), in the layouts of prob.geom: metrics_vc (n_volumes, n_vc, d, d), jacobian_det_vc
    (n_volumes, n_vc), normals_fc (n_faces, n_fc, d), jacobian_det_fc (n_faces, n_fc), xyz_fc (n_faces, n_fc, d)."""
    lib = _lib.load()
    ops, mesh, d = prob.ops, prob.mesh, prob.d
    w = np.ascontiguousarray(ops.w_vc_1d, dtype=np.float64)
    tp = _lib.TPOperators()
    tp.elem_type, tp.p, tp.w_vc = ops.e_type, ops.p, _dp(w)
    gc = _geom_coef(prob)
    fv = np.ascontiguousarray(mesh.face_vol, dtype=np.int32)
    flf = np.ascontiguousarray(mesh.face_lf, dtype=np.int32)
    m = _lib.Mesh()
    m.n_volumes, m.n_faces = mesh.n_volumes, mesh.n_faces
    m.face_vol, m.face_lf = _ip(fv), _ip(flf)
    m.p_g, m.geom_coef = prob.geom.p_g, _dp(gc)
    nv, nf, nc, nfc = mesh.n_volumes, mesh.n_faces, ops.n_vc, ops.n_fc
    met = np.empty((nv, d, d, nc))          # [v][j][i][c]: column-major (n_vc, d, d)
    jac = np.empty((nv, nc))
    nrm = np.empty((nf, nfc, d))
    jf = np.empty((nf, nfc))
    xyz = np.empty((nf, nfc, d))
    check(lib.dgpu_compute_geometry(d, ctypes.byref(tp), ctypes.byref(m), _dp(met), _dp(jac), _dp(nrm), _dp(jf),
                                    _dp(xyz)), None)
    return {"metrics_vc": np.transpose(met, (0, 3, 2, 1)), "jacobian_det_vc": jac, "normals_fc": nrm,
            "jacobian_det_fc": jf, "xyz_fc": xyz}


class Simulation:
    """One dgpu context for a TP DGProblem (dpgsolver_gb300.host.problem). device_geometry=True hands the library
    the geometry coefficients instead of the host's geometric factors, and the device computes them."""

    def __init__(self, prob, stream=None, device_geometry=False):
        lib = _lib.load()
        ops, mesh, geom = prob.ops, prob.mesh, prob.geom
        d = prob.d
        self._keep = keep = {}

        def arr(name, a, dtype=np.float64):
            keep[name] = np.ascontiguousarray(a, dtype=dtype)
            return keep[name]

        phys = _lib.Physics()
        phys.d, phys.pde, phys.num_flux = d, prob.pde, prob.num_flux
        phys.positivity = 1 if prob.positivity else 0
        for k in range(3):
            phys.b_adv[k] = float(prob.b_adv[k])
        ns = getattr(prob, "ns", None)
        if ns is not None:
            phys.viscosity, phys.mu, phys.Pr, phys.r_s = int(ns["viscosity"]), ns["mu"], ns["Pr"], ns["r_s"]
            phys.dTdn = float(ns.get("dTdn", 0.0))
        tp = _lib.TPOperators()
        tp.elem_type = ops.e_type
        tp.p = ops.p
        tp.cv0_vs_vc = _dp(arr("cv0", ops.cv0_1d))
        tp.cv1_vs_vc = _dp(arr("cv1", ops.cv1_1d))
        tp.cv0_vs_fc = _dp(arr("cv0f", ops.cv0_bnd_1d))
        tp.w_vc = _dp(arr("w", ops.w_vc_1d))
        tp.ccSB0_vs_vs = _dp(arr("sb", ops.ccSB0_1d))
        tp.ccBS0_vs_vs = _dp(arr("bs", ops.ccBS0_1d))
        m = _lib.Mesh()
        m.n_volumes = mesh.n_volumes
        if device_geometry:
            m.p_g = geom.p_g
            m.geom_coef = _dp(arr("gc", _geom_coef(prob)))
        else:
            m.metrics_vc = _dp(arr("m", np.transpose(geom.metrics_vc, (0, 3, 2, 1))))
            m.jacobian_det_vc = _dp(arr("J", geom.jacobian_det_vc))
        m.n_faces = mesh.n_faces
        m.face_vol = _ip(arr("fv", mesh.face_vol, np.int32))
        m.face_lf = _ip(arr("flf", mesh.face_lf, np.int32))
        nc = prob.nc_fc()
        m.nc_fc = _ip(arr("nc", nc, np.int32))
        if not device_geometry:
            m.normals_fc = _dp(arr("nrm", geom.normals_fc))
            m.jacobian_det_fc = _dp(arr("Jf", geom.jacobian_det_fc))
        if getattr(prob, "bc", None) is not None:
            if np.size(prob.bc) != mesh.n_faces or np.size(prob.bc_state) != mesh.n_faces * ops.n_fc * prob.n_var:
                raise ValueError("bc needs one code per face and bc_state (n_faces, n_fc, n_var) values")
            m.bc_fc = _ip(arr("bc", prob.bc, np.int32))
            m.bc_state_fc = _dp(arr("bcs", prob.bc_state))
            if getattr(prob, "bc_data", None) is not None:
                m.bc_data = _dp(arr("bcd", np.asarray(prob.bc_data, dtype=np.float64).reshape(4)))
        h = ctypes.c_void_p()
        st = lib.dgpu_create(ctypes.byref(phys), ctypes.byref(tp), ctypes.byref(m), ctypes.byref(h))
        check(st, None)
        self._lib = lib
        self._h = h
        self._keep = {}  # the library copied everything
        self.prob = prob
        self.shape = prob.sol.shape
        if stream is not None:
            check(lib.dgpu_set_stream(h, ctypes.c_void_p(stream)), h)
        self.upload_state(prob.sol)
        if getattr(prob, "source_vc", None) is not None:
            self.set_source(prob.source_vc)

    # -- lifetime ------------------------------------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.dgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- state ---------------------------------------------------------------------------------------------------
    def upload_state(self, sol):
        s = np.ascontiguousarray(sol, dtype=np.float64)
        if s.shape != self.shape:
            raise ValueError(f"state shape {s.shape} != {self.shape}")
        check(self._lib.dgpu_upload_state(self._h, _dp(s)), self._h)

    @property
    def sol_coef(self):
        out = np.empty(self.shape)
        check(self._lib.dgpu_download_state(self._h, _dp(out)), self._h)
        return out

    @property
    def rhs(self):
        out = np.empty(self.shape)
        check(self._lib.dgpu_download_rhs(self._h, _dp(out)), self._h)
        return out

    # -- compute -------------------------------------------------------------------------------------------------
    def set_source(self, source_vc):
        """The test case's source at the volume cubature nodes, in the state's shape (None removes it)."""
        if source_vc is None:
            check(self._lib.dgpu_set_source(self._h, None), self._h)
            return
        s = np.ascontiguousarray(source_vc, dtype=np.float64)
        if s.shape != self.shape:
            raise ValueError(f"source shape {s.shape} != {self.shape}")
        check(self._lib.dgpu_set_source(self._h, _dp(s)), self._h)

    def compute_rhs(self, want_max: bool = True):
        mx = ctypes.c_double()
        check(self._lib.dgpu_compute_rhs(self._h, ctypes.byref(mx) if want_max else None), self._h)
        return mx.value if want_max else None

    def compute_rhs_host(self, sol, out=None):
        s = np.ascontiguousarray(sol, dtype=np.float64)
        r = out if out is not None else np.empty(self.shape)
        mx = ctypes.c_double()
        check(self._lib.dgpu_compute_rhs_host(self._h, _dp(s), _dp(r), ctypes.byref(mx)), self._h)
        return r, mx.value

    def ssp_rk3_steps(self, dt: float, n_steps: int = 1, want_max: bool = True):
        mx = ctypes.c_double()
        check(self._lib.dgpu_ssp_rk3_steps(self._h, float(dt), int(n_steps), ctypes.byref(mx) if want_max else None),
              self._h)
        return mx.value if want_max else None

    # -- discrete adjoint (autograd-Function-shaped pair) ------------------------------------------------------
    def vjp_forward(self, sol):
        """R(sol) (compute_rhs_dg on host buffers); keeps sol for vjp_backward. Returns (rhs, max_rhs)."""
        s = np.ascontiguousarray(sol, dtype=np.float64)
        r = np.empty(self.shape)
        mx = ctypes.c_double()
        check(self._lib.dgpu_vjp_forward(self._h, _dp(s), _dp(r), ctypes.byref(mx)), self._h)
        return r, mx.value

    def jvp(self, sol, direction):
        """(R(sol), (dR/dsol) direction) by forward mode (dual numbers through the flux routines)."""
        s = np.ascontiguousarray(sol, dtype=np.float64)
        d = np.ascontiguousarray(direction, dtype=np.float64)
        if s.shape != self.shape or d.shape != self.shape:
            raise ValueError(f"state shape {s.shape} / {d.shape} != {self.shape}")
        r = np.empty(self.shape)
        jv = np.empty(self.shape)
        check(self._lib.dgpu_jvp(self._h, _dp(s), _dp(d), _dp(r), _dp(jv)), self._h)
        return r, jv

    def jacobian_structure(self):
        """(block_size, n_blocks, n_colours) of the block-sparse Jacobian (dgpu_jacobian_structure)."""
        nb, nnz, nc = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_int()
        check(self._lib.dgpu_jacobian_structure(self._h, ctypes.byref(nb), ctypes.byref(nnz), ctypes.byref(nc)),
              self._h)
        return nb.value, nnz.value, nc.value

    def jacobian(self, sol, raw=True, values_ptr=None):
        """Block-sparse Jacobian at sol (dgpu_jacobian_bsr): (row_ptr, col_idx, values) with values
        (n_blocks, block_size, block_size), row-major blocks in the reference's lhs layout. raw: of the residual
        before M^-1 (the reference's lhs) or of the explicit right-hand side. values_ptr: a device address of
        n_blocks * block_size^2 doubles to write the blocks to instead (values is then None)."""
        s = np.ascontiguousarray(sol, dtype=np.float64)
        if s.shape != self.shape:
            raise ValueError(f"state shape {s.shape} != {self.shape}")
        nb, nnz, _ = self.jacobian_structure()
        row_ptr = np.empty(self.prob.n_volumes + 1, dtype=np.int32)
        col_idx = np.empty(nnz, dtype=np.int32)
        vals = None if values_ptr is not None else np.empty((nnz, nb, nb))
        ptr = ctypes.c_void_p(values_ptr) if values_ptr is not None else vals.ctypes.data_as(ctypes.c_void_p)
        check(self._lib.dgpu_jacobian_bsr(self._h, _dp(s), 1 if raw else 0, _ip(row_ptr), _ip(col_idx), ptr),
              self._h)
        return row_ptr, col_idx, vals

    def vjp_backward(self, cotangent):
        """(dR/dsol)^T cotangent at the state kept by vjp_forward."""
        v = np.ascontiguousarray(cotangent, dtype=np.float64)
        if v.shape != self.shape:
            raise ValueError(f"cotangent shape {v.shape} != {self.shape}")
        g = np.empty(self.shape)
        check(self._lib.dgpu_vjp_backward(self._h, _dp(v), _dp(g)), self._h)
        return g

    def set_objective_faces(self, faces):
        f = np.ascontiguousarray(faces, dtype=np.int32)
        check(self._lib.dgpu_set_objective_faces(self._h, int(f.size), _ip(f)), self._h)

    def objective(self, sol, gradient: bool = True):
        """J(sol) = integral of pressure over the objective faces (side 0) and dJ/dsol."""
        s = np.ascontiguousarray(sol, dtype=np.float64)
        J = ctypes.c_double()
        g = np.empty(self.shape) if gradient else None
        check(self._lib.dgpu_objective(self._h, _dp(s), ctypes.byref(J), _dp(g) if gradient else None), self._h)
        return (J.value, g) if gradient else J.value

    def adjoint_ssp_rk3(self, sol0, dt: float, n_steps: int, budget_bytes: int):
        """J(sol after n_steps SSP-RK3 steps) and dJ/dsol0, with checkpointed recomputation in budget_bytes."""
        s = np.ascontiguousarray(sol0, dtype=np.float64)
        J = ctypes.c_double()
        g = np.empty(self.shape)
        K = ctypes.c_int()
        check(self._lib.dgpu_adjoint_ssp_rk3(self._h, float(dt), int(n_steps), int(budget_bytes), _dp(s),
                                             ctypes.byref(J), _dp(g), ctypes.byref(K)), self._h)
        return J.value, g, K.value

    def synchronize(self):
        check(self._lib.dgpu_synchronize(self._h), self._h)

    def positivity_corrections(self) -> int:
        n = ctypes.c_longlong()
        check(self._lib.dgpu_positivity_corrections(self._h, ctypes.byref(n)), self._h)
        return n.value

    def kernel_launches(self) -> int:
        n = ctypes.c_longlong()
        check(self._lib.dgpu_kernel_launches(self._h, ctypes.byref(n)), self._h)
        return n.value

    def set_kernel_timing(self, enable: bool):
        check(self._lib.dgpu_set_kernel_timing(self._h, 1 if enable else 0), self._h)

    def kernel_time(self, name: str):
        tot = ctypes.c_double()
        cnt = ctypes.c_longlong()
        check(self._lib.dgpu_kernel_time(self._h, name.encode(), ctypes.byref(tot), ctypes.byref(cnt)), self._h)
        return tot.value, cnt.value


class BatchSimulation:
    """One batched dgpu context for a mixed-order TP mesh (dpgsolver_gb300.host.mixed.MixedTPProblem, or a uniform
    DGProblem as a one-group mesh). States are flat arrays in volume-list order (the problem's layout)."""

    def __init__(self, prob, stream=None, factorised: bool = True):
        """factorised: pass the TRI x LINE factors of WEDGE groups (sum-factorised volume term); False runs every
        TET/WEDGE/PYR group through the dense per-volume products."""
        from .host.problem import flat_arrays

        lib = _lib.load()
        fl = flat_arrays(prob)
        d = prob.d
        keep = []

        def arr(a, dtype=np.float64):
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return a

        phys = _lib.Physics()
        phys.d, phys.pde, phys.num_flux = d, prob.pde, prob.num_flux
        phys.positivity = 1 if prob.positivity else 0
        for k in range(3):
            phys.b_adv[k] = float(prob.b_adv[k])
        ns = getattr(prob, "ns", None)
        if ns is not None:
            phys.viscosity, phys.mu, phys.Pr, phys.r_s = int(ns["viscosity"]), ns["mu"], ns["Pr"], ns["r_s"]
            phys.dTdn = float(ns.get("dTdn", 0.0))
        groups = fl["groups"]
        dense = any(getattr(o, "dense", False) for o in groups)
        tps = (_lib.TPOperators * len(groups))()
        dns = (_lib.DenseOperators * len(groups))()
        for g, ops in enumerate(groups):
            if getattr(ops, "dense", False):
                self._dense_operators(dns[g], ops, arr, keep, factorised)
                continue
            tps[g].elem_type, tps[g].p = ops.e_type, ops.p
            tps[g].cv0_vs_vc = _dp(arr(ops.cv0_1d))
            tps[g].cv1_vs_vc = _dp(arr(ops.cv1_1d))
            tps[g].cv0_vs_fc = _dp(arr(ops.cv0_bnd_1d))
            tps[g].w_vc = _dp(arr(ops.w_vc_1d))
            tps[g].ccSB0_vs_vs = _dp(arr(ops.ccSB0_1d))
            tps[g].ccBS0_vs_vs = _dp(arr(ops.ccBS0_1d))
        mesh = prob.mesh
        m = _lib.Mesh()
        m.n_volumes = mesh.n_volumes
        m.metrics_vc = _dp(arr(fl["metrics_vc"]))
        m.jacobian_det_vc = _dp(arr(fl["jacobian_det_vc"]))
        m.n_faces = mesh.n_faces
        m.face_vol = _ip(arr(mesh.face_vol, np.int32))
        m.face_lf = _ip(arr(mesh.face_lf, np.int32))
        m.nc_fc = _ip(arr(fl["nc_fc"], np.int32))
        m.normals_fc = _dp(arr(fl["normals_fc"]))
        m.jacobian_det_fc = _dp(arr(fl["jacobian_det_fc"]))
        if fl.get("bc_fc") is not None:
            m.bc_fc = _ip(arr(fl["bc_fc"], np.int32))
            m.bc_state_fc = _dp(arr(fl["bc_state_fc"]))
            if fl.get("bc_data") is not None:
                m.bc_data = _dp(arr(np.asarray(fl["bc_data"], dtype=np.float64).reshape(4)))
        vg = arr(fl["vol_group"], np.int32)
        h = ctypes.c_void_p()
        if dense or fl.get("face_ord") is not None:
            G = (_lib.Group * len(groups))()
            for g, ops in enumerate(groups):
                if getattr(ops, "dense", False):
                    G[g].dense = ctypes.pointer(dns[g])
                else:
                    G[g].tp = ctypes.pointer(tps[g])
            fo = fl.get("face_ord")
            fop = _ip(arr(fo, np.int32)) if fo is not None else None
            check(lib.dgpu_batch_create_groups(ctypes.byref(phys), len(groups), G, _ip(vg), ctypes.byref(m), fop,
                                               ctypes.byref(h)), None, batch=True)
        else:
            check(lib.dgpu_batch_create(ctypes.byref(phys), len(groups), tps, _ip(vg), ctypes.byref(m),
                                        ctypes.byref(h)), None, batch=True)
        self._lib = lib
        self._h = h
        self.prob = prob
        n = ctypes.c_size_t()
        check(lib.dgpu_batch_state_size(h, ctypes.byref(n)), h, batch=True)
        self.n_state = n.value
        self.shape = np.shape(fl["sol"]) if np.ndim(prob.sol) == 1 else prob.sol.shape
        if stream is not None:
            check(lib.dgpu_batch_set_stream(h, ctypes.c_void_p(stream)), h, batch=True)
        self.upload_state(prob.sol)
        n_vc = np.array([int(o.n_vc) for o in groups], dtype=np.int64)
        self._n_source = int(n_vc[np.asarray(fl["vol_group"])].sum()) * int(prob.n_var)
        if getattr(prob, "source_vc", None) is not None:
            self.set_source(prob.source_vc)

    @staticmethod
    def _dense_operators(D, ops, arr, keep, factorised=True):
        """Fill a DenseOperators struct from a DenseOperatorSet: volume operators and the face operator table for
        every local face, orientation and face order p_f >= p."""
        from .host import simplex as S
        n_ord = 8
        D.elem_type, D.p, D.n_vs, D.n_vc = ops.e_type, ops.p, ops.n_vs, ops.n_vc
        D.cv0_vs_vc = _dp(arr(ops.cv0_vs_vc()))
        D.cv1_vs_vc = _dp(arr(np.stack([ops.cv1_vs_vc(k) for k in range(ops.d)])))
        D.w_vc = _dp(arr(ops.w_vc))
        D.n_lf, D.n_ord = ops.n_lf, n_ord
        n_fc = np.zeros(ops.n_lf * n_ord * 5, dtype=np.int32)
        cv0 = (_lib.c_double_p * (ops.n_lf * n_ord * 5))()
        w = (_lib.c_double_p * (ops.n_lf * 5))()
        for lf in range(ops.n_lf):
            for pf in range(ops.p, 5):
                w[lf * 5 + pf] = _dp(arr(ops.w_fc(lf, pf + 1)))
                for o in range(ops.n_ords(lf)):
                    c = arr(ops.cv0_vs_fc(lf, o, pf + 1))
                    n_fc[(lf * n_ord + o) * 5 + pf] = c.shape[0]
                    cv0[(lf * n_ord + o) * 5 + pf] = _dp(c)
        D.n_fc = _ip(arr(n_fc, np.int32))
        D.cv0_vs_fc = cv0
        D.w_fc = w
        keep.extend([cv0, w])
        D.ccSB0_vs_vs = _dp(arr(ops.ccSB0_vs_vs()))
        D.ccBS0_vs_vs = _dp(arr(ops.ccBS0_vs_vs()))
        if ops.e_type == S.WEDGE and factorised:
            t0, t1, l0, l1 = ops.prism_factors()
            D.n_tri_vs, D.n_tri_vc = t0.shape[1], t0.shape[0]
            D.n_line_vs, D.n_line_vc = l0.shape[1], l0.shape[0]
            D.tri_cv0, D.tri_cv1 = _dp(arr(t0)), _dp(arr(t1))
            D.line_cv0, D.line_cv1 = _dp(arr(l0)), _dp(arr(l1))

    def _check(self, st):
        check(st, self._h, batch=True)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.dgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload_state(self, sol):
        s = np.ascontiguousarray(sol, dtype=np.float64)
        if s.size != self.n_state:
            raise ValueError(f"state has {s.size} values, the mesh {self.n_state}")
        self._check(self._lib.dgpu_batch_upload_state(self._h, _dp(s)))

    @property
    def sol_coef(self):
        out = np.empty(self.shape)
        self._check(self._lib.dgpu_batch_download_state(self._h, _dp(out)))
        return out

    @property
    def rhs(self):
        out = np.empty(self.shape)
        self._check(self._lib.dgpu_batch_download_rhs(self._h, _dp(out)))
        return out

    def compute_rhs(self, want_max: bool = True):
        mx = ctypes.c_double()
        self._check(self._lib.dgpu_batch_compute_rhs(self._h, ctypes.byref(mx) if want_max else None))
        return mx.value if want_max else None

    def ssp_rk3_steps(self, dt: float, n_steps: int = 1, want_max: bool = True):
        mx = ctypes.c_double()
        self._check(self._lib.dgpu_batch_ssp_rk3_steps(self._h, float(dt), int(n_steps),
                                                       ctypes.byref(mx) if want_max else None))
        return mx.value if want_max else None

    def set_source(self, source_vc):
        """The test case's source at every volume's cubature nodes (flat, volume-list order, per volume
        (n_var x n_vc) blocks as the reference's column-major (n_vc x n_var)), or None to remove it."""
        if source_vc is None:
            self._check(self._lib.dgpu_batch_set_source(self._h, None))
            return
        s = np.ascontiguousarray(source_vc, dtype=np.float64).ravel()
        if s.size != self._n_source:
            raise ValueError(f"source of {s.size} values, expected {self._n_source}")
        self._check(self._lib.dgpu_batch_set_source(self._h, _dp(s)))

    def set_barrier_timeout(self, seconds: float):
        """Bound of each grid-barrier wait of the "stage" form (2 s by default)."""
        self._check(self._lib.dgpu_batch_set_barrier_timeout(self._h, float(seconds)))

    FORMS = {"plain": 0, "fused": 1, "branches": 2, "stage": 3}

    @property
    def form(self) -> str:
        """Launch form of the stages: "plain" (one launch per group / face order), "fused" (persistent launches
        over all groups), "branches" (the plain launches on parallel graph branches) or "stage" (the whole stage
        in one cooperative persistent launch)."""
        v = ctypes.c_int()
        self._check(self._lib.dgpu_batch_get_mode(self._h, ctypes.byref(v)))
        return {v: k for k, v in self.FORMS.items()}[v.value]

    @form.setter
    def form(self, name: str):
        self._check(self._lib.dgpu_batch_set_mode(self._h, self.FORMS[name]))

    @property
    def fused(self) -> bool:
        return self.form == "fused"

    @fused.setter
    def fused(self, on: bool):
        self.form = "fused" if on else "plain"

    def set_graphs(self, enable: bool):
        """Replay RK steps from a captured CUDA graph (default) or launch every kernel from the host."""
        self._check(self._lib.dgpu_batch_set_graphs(self._h, 1 if enable else 0))

    def set_group_tile(self, group: int, elements_per_cta: int):
        self._check(self._lib.dgpu_batch_set_group_tile(self._h, int(group), int(elements_per_cta)))

    def autotune(self, dt: float, reps: int = 3) -> str:
        buf = ctypes.create_string_buffer(8192)
        self._check(self._lib.dgpu_batch_autotune(self._h, float(dt), int(reps), buf, len(buf)))
        return buf.value.decode()

    def kernel_launches(self) -> int:
        n = ctypes.c_longlong()
        self._check(self._lib.dgpu_batch_kernel_launches(self._h, ctypes.byref(n)))
        return n.value

    def positivity_corrections(self) -> int:
        n = ctypes.c_longlong()
        self._check(self._lib.dgpu_batch_positivity_corrections(self._h, ctypes.byref(n)))
        return n.value


class _DeviceArray:
    """__cuda_array_interface__ view of a device buffer the library owns (for torch.as_tensor, zero copy)."""

    def __init__(self, ptr: int, shape):
        self.__cuda_array_interface__ = {"shape": tuple(int(x) for x in shape), "typestr": "<f8",
                                         "data": (int(ptr), False), "version": 3}


class PartitionSimulation(Simulation):
    """One rank's share of an element-partitioned mesh (dpgsolver_gb300.partition.Partition) on this process's GPU:
    a dgpu context on the rank's volumes and faces, the halo plan (dgpu_halo_setup), and the residual / SSP-RK3
    stages split around the exchange of the cut faces' traces (dgpu_halo_*_begin / _end). The whole-mesh calls of
    Simulation (compute_rhs, ssp_rk3_steps, ...) are refused by the library on such a context."""

    def __init__(self, prob, part, stream=None):
        super().__init__(part.local_problem(prob), stream=stream)
        self.part = part
        send = np.ascontiguousarray(part.send_slots, dtype=np.int32)
        recv = np.ascontiguousarray(part.recv_slots, dtype=np.int32)
        check(self._lib.dgpu_halo_setup(self._h, len(send), _ip(send), _ip(recv)), self._h)
        ps, pr, sd = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_size_t()
        check(self._lib.dgpu_halo_buffers(self._h, ctypes.byref(ps), ctypes.byref(pr), ctypes.byref(sd)), self._h)
        st = ctypes.c_void_p()
        check(self._lib.dgpu_get_stream(self._h, ctypes.byref(st)), self._h)
        self.slot_doubles = sd.value
        self._send_ptr, self._recv_ptr, self.stream_ptr = ps.value, pr.value, st.value

    def halo_tensors(self):
        """(send, recv) torch views (n_halo, slot_doubles) of the library's halo buffers, for NCCL or copies; None
        when this rank has no cut face."""
        import torch
        n = self.part.n_halo
        if n == 0:
            return None, None
        shape = (n, self.slot_doubles)
        return (torch.as_tensor(_DeviceArray(self._send_ptr, shape), device="cuda"),
                torch.as_tensor(_DeviceArray(self._recv_ptr, shape), device="cuda"))

    def rhs_begin(self):
        check(self._lib.dgpu_halo_rhs_begin(self._h), self._h)

    def rhs_end(self, want_max: bool = True):
        mx = ctypes.c_double()
        check(self._lib.dgpu_halo_rhs_end(self._h, ctypes.byref(mx) if want_max else None), self._h)
        return mx.value if want_max else None

    def stage_begin(self, stage: int):
        check(self._lib.dgpu_halo_stage_begin(self._h, int(stage)), self._h)

    def stage_end(self, dt: float, stage: int, want_max: bool = False):
        mx = ctypes.c_double()
        check(self._lib.dgpu_halo_stage_end(self._h, float(dt), int(stage), ctypes.byref(mx) if want_max else None),
              self._h)
        return mx.value if want_max else None


def compute_rhs_dg(sim: Simulation) -> float:
    """compute_rhs_dg (solvers/dg/solve_dg.c:130-136): residual of sim's state into sim's rhs; max |rhs|."""
    return sim.compute_rhs()


def time_step_ssp_rk_33(dt: float, sim: Simulation) -> float:
    """time_step_ssp_rk_33 (solvers/solve_explicit.c:252-301): one SSP-RK3 step; max |rhs| of the last stage."""
    return sim.ssp_rk3_steps(dt, 1)


def solve_explicit(sim: Simulation, n_steps: int, dt: float | None = None) -> float:
    """The explicit time loop (solvers/solve_explicit.c:78-118) for a fixed number of steps."""
    return sim.ssp_rk3_steps(sim.prob.dt if dt is None else dt, n_steps)
