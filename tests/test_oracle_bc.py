"""The CPU oracle on bounded domains: boundary faces with the reference's BC codes (definitions_bc.h).

Known-answer properties of the boundary values (test_case/boundary/boundary_euler_T.c, boundary_advection_T.c):
a stream that satisfies every boundary condition is preserved; slip walls carry no mass; the advection residual of
a smooth field with the exact field as exterior state converges spectrally up to the boundary; the complex
instantiation of every boundary value differentiates it.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import problem as P


def _stream(prob, rho, vel, p):
    d = prob.d
    vel = np.asarray(vel, dtype=np.float64)
    E = p / P.GM1 + 0.5 * rho * float(vel @ vel)
    return P.constant_state(prob, [rho] + list(rho * vel) + [E])


def _exterior(prob, rho, vel, p):
    U = _stream(prob, rho, vel, p)[0, :, 0]
    prob.bc_state = np.where((prob.mesh.face_vol[:, 1] < 0)[:, None, None], U[None, None, :], 0.0) \
        * np.ones_like(prob.bc_state)
    return prob


@pytest.mark.parametrize("flux", [P.NUM_FLUX_LAX_FRIEDRICHS, P.NUM_FLUX_ROE_PIKE])
def test_riemann_boundaries_preserve_free_stream(flux):
    """All four sides BC_RIEMANN with the free stream as exterior: the constant stream is a steady state on the
    curved mesh (subsonic inflow and outflow sides both appear)."""
    prob = P.euler_riemann_2d(5, 3, num_flux=flux)
    _, mx = oracle.Oracle(prob).compute_rhs(_stream(prob, 1.0, (1.0, 1.0), 1.0))
    assert mx < 1e-11


def test_slip_walls_preserve_tangential_stream():
    """Slip walls at y = 0 and y = 10 (straight under the sinusoidal mapping): a stream along x is steady."""
    prob = P.euler_channel_2d(5, 3)
    _, mx = oracle.Oracle(prob).compute_rhs(_stream(prob, 1.0, (0.8, 0.0), 1.0))
    assert mx < 1e-11


@pytest.mark.parametrize("flux", [P.NUM_FLUX_LAX_FRIEDRICHS, P.NUM_FLUX_ROE_PIKE])
def test_duct_preserves_supersonic_stream(flux):
    """Supersonic inflow/outflow in x, slip walls in y, Riemann in z, the Mach 2 stream as exterior."""
    prob = P.euler_duct_3d(3, 2, num_flux=flux)
    u0 = 2.0 * np.sqrt(P.GAMMA)
    _, mx = oracle.Oracle(prob).compute_rhs(_stream(prob, 1.0, (u0, 0.0, 0.0), 1.0))
    assert mx < 1e-10


def test_riemann_subsonic_outflow_and_inflow_states():
    """A stream different from the exterior one: the residual is not zero, the boundary state being built from
    the outgoing invariant of the interior and the incoming one of the exterior."""
    prob = _exterior(P.euler_riemann_2d(4, 2), 1.0, (0.3, 0.1), 1.0)
    o = oracle.Oracle(prob)
    _, mx0 = o.compute_rhs(_stream(prob, 1.0, (0.3, 0.1), 1.0))
    _, mx1 = o.compute_rhs(_stream(prob, 1.1, (0.3, 0.1), 1.0))
    assert mx0 < 1e-11 and mx1 > 1e-3


def test_slip_walls_conserve_mass():
    """Periodic in x, slip walls in y, Lax-Friedrichs: the mirror state makes the wall mass flux vanish, so the raw
    residual's mass total telescopes to zero."""
    prob = P.euler_channel_2d(5, 3, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS)
    raw = oracle.Oracle(prob).compute_rhs_raw(prob.sol)
    assert abs(raw[:, 0].sum()) <= 1e-13 * np.abs(raw[:, 0]).sum()


def test_advection_box_residual_converges_at_the_boundary():
    """Upwind boundaries with the exact field as exterior: the residual approximates -b.grad(u) spectrally in
    every element, the boundary elements included."""
    errs = []
    for n in (4, 8):
        prob = P.advection_box_2d(n, 3)
        r, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
        xyz = prob.solution_node_xyz()
        x, y = xyz[..., 0], xyz[..., 1]
        exact = -(np.pi * np.cos(np.pi * x) * np.sin(np.pi * y) + 0.5 * np.pi * np.sin(np.pi * x) * np.cos(np.pi * y))
        errs.append(np.max(np.abs(r[:, 0, :] - exact)))
    assert errs[1] < errs[0] / 6.0


def test_advection_box_inflow_takes_exterior_state():
    """Raising the exterior state changes the residual only in the elements on the inflow sides (x = -1, y = -1
    for b = (1, 0.5))."""
    prob = P.advection_box_2d(4, 2)
    r0, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    prob.bc_state = prob.bc_state + 1.0
    r1, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    changed = np.abs(r1 - r0).max(axis=(1, 2)) > 1e-12
    ijk = prob.mesh.ijk
    inflow = (ijk[:, 0] == 0) | (ijk[:, 1] == 0)
    assert np.array_equal(changed, inflow)


@pytest.mark.parametrize("mk", [lambda: P.euler_riemann_2d(3, 2, num_flux=P.NUM_FLUX_ROE_PIKE),
                                lambda: P.euler_channel_2d(3, 2), lambda: P.euler_duct_3d(2, 2)])
def test_boundary_complex_step(mk):
    """The complex instantiation of the boundary values (the reference's complex-step linearisation) agrees with
    central differences."""
    prob = mk()
    o = oracle.Oracle(prob)
    rng = np.random.default_rng(3)
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    dirn = rng.standard_normal(prob.sol.shape)
    h = 1e-30
    _, ri = o.compute_rhs_cmplx(base, h * dirn)
    jv_cs = ri / h
    eps = 1e-6
    rp, _ = o.compute_rhs(base + eps * dirn)
    rm, _ = o.compute_rhs(base - eps * dirn)
    assert np.max(np.abs(jv_cs - (rp - rm) / (2 * eps))) <= 1e-6 * np.max(np.abs(jv_cs))


def test_boundary_face_needs_bc_arrays():
    prob = P.euler_channel_2d(3, 2)
    prob.bc = None
    prob.bc_state = None
    with pytest.raises(Exception):
        oracle.Oracle(prob)


def test_unknown_bc_code_is_an_error():
    prob = P.euler_channel_2d(3, 2)
    prob.bc = np.where(prob.bc > 0, 111, 0).astype(np.int32)   # BC_NOSLIP_ADIABATIC: Navier-Stokes only
    with pytest.raises(Exception):
        oracle.Oracle(prob).compute_rhs(prob.sol)


@pytest.mark.parametrize("mk,sides", [
    (lambda: P.euler_channel_2d(4, 2), {(1, 0): 102, (1, 1): 102}),
    (lambda: P.euler_duct_3d(3, 2), {(0, 0): 105, (0, 1): 106, (1, 0): 102, (1, 1): 102, (2, 0): 101, (2, 1): 101}),
    (lambda: P.advection_box_2d(3, 2), {(0, 0): 41, (0, 1): 41, (1, 0): 41, (1, 1): 41})])
def test_boundary_layout(mk, sides):
    """Every boundary face carries its side's code and an exterior state per face node; interior faces carry 0,
    and the boundary faces' normals point out of the domain."""
    prob = mk()
    m = prob.mesh
    bnd = m.face_vol[:, 1] < 0
    assert np.all(m.face_lf[bnd, 1] == -1) and np.all(prob.bc[~bnd] == 0)
    for f in np.nonzero(bnd)[0]:
        lf = int(m.face_lf[f, 0])
        assert prob.bc[f] == sides[(lf // 2, lf % 2)]
        nrm = prob.geom.normals_fc[f]
        assert np.all(nrm[:, lf // 2] * (1 if lf % 2 else -1) > 0.5)
    assert prob.bc_state.shape == (m.n_faces, prob.ops.n_fc, prob.n_var)
    assert set(map(tuple, np.unique(np.stack([m.face_lf[bnd, 0] // 2, m.face_lf[bnd, 0] % 2], 1), axis=0))) \
        == set(sides)


@pytest.mark.parametrize("d,flux", [(2, P.NUM_FLUX_ROE_PIKE), (2, P.NUM_FLUX_LAX_FRIEDRICHS), (3, P.NUM_FLUX_ROE_PIKE)])
def test_total_tp_and_back_pressure_preserve_their_stream(d, flux):
    """Total temperature/pressure inflow and back-pressure outflow whose data come from a subsonic stream along x
    (slip walls elsewhere): that stream is steady."""
    prob = P.euler_subsonic_duct(d, 3, 2, num_flux=flux)
    u0 = 0.4 * np.sqrt(P.GAMMA)
    _, mx = oracle.Oracle(prob).compute_rhs(_stream(prob, 1.0, (u0,) + (0.0,) * (d - 1), 1.0))
    assert mx < 1e-10


def test_back_pressure_sets_the_outflow_pressure():
    """Raising p_back changes the residual only in the elements at the outflow end x = 10."""
    prob = P.euler_subsonic_duct(2, 4, 2)
    r0, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    prob.bc_data = (1.2,) + tuple(prob.bc_data[1:])
    r1, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    changed = np.abs(r1 - r0).max(axis=(1, 2)) > 1e-12
    assert np.array_equal(changed, prob.mesh.ijk[:, 0] == 3)


def test_total_tp_and_back_pressure_complex_step():
    prob = P.euler_subsonic_duct(2, 3, 2)
    o = oracle.Oracle(prob)
    rng = np.random.default_rng(5)
    base = prob.sol + 1e-2 * rng.standard_normal(prob.sol.shape)
    dirn = rng.standard_normal(prob.sol.shape)
    _, ri = o.compute_rhs_cmplx(base, 1e-30 * dirn)
    eps = 1e-6
    rp, _ = o.compute_rhs(base + eps * dirn)
    rm, _ = o.compute_rhs(base - eps * dirn)
    jv = ri / 1e-30
    assert np.max(np.abs(jv - (rp - rm) / (2 * eps))) <= 1e-6 * np.max(np.abs(jv))
