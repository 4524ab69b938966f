"""State transfers between the caller's host buffers and a context (dgpu_upload_state / dgpu_download_state).

A page-locked buffer is read and written by the basis-change kernel directly over the host link, in place of a
copy followed by a separate conversion. The results must be bit for bit those of the pageable path (copy, then the
same conversion kernel).
"""
import ctypes

import numpy as np
import pytest

from dpgsolver_gb300 import _lib
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mk", [lambda: P.euler_hex_3d(4, 3), lambda: P.euler_vortex_2d(6, 2),
                                lambda: P.advection_2d(8, 2), lambda: P.ns_taylor_green(3, 2, mach=0.3)])
def test_pinned_and_pageable_transfers_agree(gpu_lib, mk):
    import torch
    from dpgsolver_gb300.solver import Simulation
    prob = mk()
    lib = _lib.load()
    base = prob.sol + 1e-3 * np.random.default_rng(2).standard_normal(prob.sol.shape)
    pin_in = torch.from_numpy(base.copy()).pin_memory()
    pin_out = torch.zeros(prob.sol.shape, dtype=torch.float64).pin_memory()
    dp = ctypes.POINTER(ctypes.c_double)
    results = []
    for pinned in (False, True):
        with Simulation(prob) as sim:
            h = sim.handle
            src = ctypes.cast(pin_in.data_ptr(), dp) if pinned else np.ascontiguousarray(base).ctypes.data_as(dp)
            _lib.check(lib.dgpu_upload_state(h, src), h)
            back = np.empty_like(base)
            _lib.check(lib.dgpu_download_state(h, back.ctypes.data_as(dp)), h)   # coefficients still current
            mx = ctypes.c_double()
            _lib.check(lib.dgpu_ssp_rk3_step(h, ctypes.c_double(prob.dt), ctypes.byref(mx)), h)
            if pinned:
                _lib.check(lib.dgpu_download_state(h, ctypes.cast(pin_out.data_ptr(), dp)), h)
                out = pin_out.numpy().copy()
            else:
                out = np.empty_like(base)
                _lib.check(lib.dgpu_download_state(h, out.ctypes.data_as(dp)), h)
            sim.compute_rhs()
            results.append((back, out, mx.value, sim.rhs))
    (b0, o0, m0, r0), (b1, o1, m1, r1) = results
    assert np.array_equal(b0, base) and np.array_equal(b1, base)
    assert np.array_equal(o0, o1)
    assert m0 == m1
    assert np.array_equal(r0, r1)


def _step_host(lib, h, dt, src, dst, want_max):
    mx = ctypes.c_double()
    _lib.check(lib.dgpu_ssp_rk3_step_host(h, ctypes.c_double(dt), src, dst, ctypes.byref(mx) if want_max else None),
               h)
    return mx.value


@pytest.mark.parametrize("mk", [lambda: P.euler_hex_3d(4, 3), lambda: P.euler_channel_2d(6, 2),
                                lambda: P.advection_2d(8, 2), lambda: P.ns_channel(2, 4, 2)])
def test_step_on_host_buffers_is_the_composed_step(gpu_lib, mk):
    """dgpu_ssp_rk3_step_host == upload + step + download, bit for bit: pinned and pageable buffers, the output
    aliasing the input, two steps on one graph, then a new dt (a new capture); the device state follows."""
    import torch
    from dpgsolver_gb300.solver import Simulation
    prob = mk()
    lib = _lib.load()
    dp = ctypes.POINTER(ctypes.c_double)
    base = prob.sol + 1e-3 * np.random.default_rng(5).standard_normal(prob.sol.shape)
    dts = (prob.dt, prob.dt, 0.5 * prob.dt)
    ref, ref_mx = [], []
    with Simulation(prob) as sim:
        h, s = sim.handle, np.ascontiguousarray(base).copy()
        for k, dt in enumerate(dts):
            _lib.check(lib.dgpu_upload_state(h, s.ctypes.data_as(dp)), h)
            mx = ctypes.c_double()
            _lib.check(lib.dgpu_ssp_rk3_step(h, ctypes.c_double(dt), ctypes.byref(mx) if k != 1 else None), h)
            _lib.check(lib.dgpu_download_state(h, s.ctypes.data_as(dp)), h)
            ref.append(s.copy())
            ref_mx.append(mx.value)
    for mode in ("pinned", "pageable", "pinned_alias"):
        with Simulation(prob) as sim:
            h = sim.handle
            if mode == "pageable":
                a, b = np.ascontiguousarray(base).copy(), np.empty_like(base)
                pa, pb = a.ctypes.data_as(dp), b.ctypes.data_as(dp)
                get = lambda: b.copy()   # noqa: E731
            else:
                ta = torch.from_numpy(base.copy()).pin_memory()
                tb = ta if mode == "pinned_alias" else torch.zeros(base.shape, dtype=torch.float64).pin_memory()
                pa, pb = ctypes.cast(ta.data_ptr(), dp), ctypes.cast(tb.data_ptr(), dp)
                get = lambda: tb.numpy().copy()   # noqa: E731
            for k, dt in enumerate(dts):
                mx = _step_host(lib, h, dt, pa, pb, k != 1)
                out = get()
                assert np.array_equal(out, ref[k]), (mode, k)
                if k != 1:
                    assert mx == ref_mx[k]
                if mode == "pageable":
                    a[...] = out
                elif mode == "pinned":
                    ta.copy_(tb)
            assert np.array_equal(sim.sol_coef, ref[-1])
