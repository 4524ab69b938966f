"""Batched mixed-order context (dgpu_batch_*) against the CPU oracle on the same seeded mixed-p meshes.

Meshes carry a seeded p in 1..4 per volume; faces are integrated at p_f = max(p_L, p_R) (face_solver.c:123-132),
which the oracle does with the dense face operators of each (group, p_f) pair. Tolerance as for the uniform path:
<= 1e-12 normwise relative error. The two launch forms (one launch per group / face order, and the fused
persistent launches) and every elements-per-CTA choice run the same per-element arithmetic, so they must agree
bit for bit.
"""
import numpy as np
import pytest

import oracle
from dpgsolver_gb300.host import mixed as M
from dpgsolver_gb300.host import mixed_types as MT
from dpgsolver_gb300.host import problem as P

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel_err(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


# The Euler states are 30 % sinusoidal perturbations of the free stream: with 5 % ones the residual on these small
# volumes is a small difference of large flux terms and input rounding alone moves it by more than 1e-12
# (test_ill_conditioned_case_within_rounding_noise). Measured noise floors of the cases below: <= 4e-13.
CASES = {
    "adv2d_mixed_8": lambda: M.mixed_advection_2d(8),
    "adv2d_mixed_curved_6": lambda: M.mixed_advection_2d(6, seed=3, curved=True),
    "vortex2d_roe_mixed_8": lambda: M.mixed_vortex_2d(8),
    "vortex2d_lf_mixed_6": lambda: M.mixed_vortex_2d(6, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS, seed=5),
    "euler2d_roe_p13_10": lambda: M.mixed_euler(2, 10, p_set=(1, 3), seed=2, perturb=0.3),
    "hex_roe_mixed_4": lambda: M.mixed_euler(3, 4, perturb=0.3),
    "hex_lf_mixed_4": lambda: M.mixed_euler(3, 4, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS, seed=1, perturb=0.3),
    "hex_roe_mixed_curved_3": lambda: M.mixed_euler(3, 3, seed=2, curved=True, perturb=0.3),
    "hex_roe_p24_5": lambda: M.mixed_euler(3, 5, p_set=(2, 4), seed=4, perturb=0.3),
    # many CTAs and tiles of every order
    "hex_roe_mixed_10": lambda: M.mixed_euler(3, 10, seed=6, perturb=0.3),
}


FORMS = ["plain", "fused", "branches", "stage"]


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("form", FORMS)
def test_residual_matches_oracle(gpu_lib, name, form):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES[name]()
    r_ref, mx_ref = oracle.Oracle(prob).compute_rhs(prob.sol)
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx = sim.compute_rhs()
        r = sim.rhs
    assert rel_err(r, r_ref) <= TOL
    assert abs(mx - mx_ref) <= TOL * mx_ref


@pytest.mark.parametrize("name,n_steps", [("adv2d_mixed_8", 4), ("vortex2d_roe_mixed_8", 3), ("hex_roe_mixed_4", 3),
                                          ("hex_lf_mixed_4", 2), ("hex_roe_mixed_curved_3", 2)])
@pytest.mark.parametrize("form", FORMS)
def test_rk3_steps_match_oracle(gpu_lib, name, n_steps, form):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES[name]()
    ref = oracle.Oracle(prob)
    s_ref = prob.sol.copy()
    for _ in range(n_steps):
        s_ref, mx_ref, _ = ref.ssp_rk3_step(s_ref, prob.dt)
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx = sim.ssp_rk3_steps(prob.dt, n_steps)
        s = sim.sol_coef
    assert rel_err(s, s_ref) <= TOL
    assert abs(mx - mx_ref) <= 1e-10 * mx_ref


# boundary faces (the reference's BCs on the ends of the non-periodic directions, exterior = the free stream)
BC_CASES = {
    "hex_roe_wall_riemann_4": lambda: M.mixed_euler(3, 4, seed=1, perturb=0.3, periodic=(True, False, True),
                                                    codes={(1, 0): 10102, (1, 1): 10101}),
    "hex_lf_supersonic_curved_3": lambda: M.mixed_euler(3, 3, seed=2, curved=True, perturb=0.3,
                                                        num_flux=P.NUM_FLUX_LAX_FRIEDRICHS,
                                                        periodic=(False, True, True),
                                                        codes={(0, 0): 10105, (0, 1): 10106}),
    "quad_roe_box_8": lambda: M.mixed_euler(2, 8, seed=3, perturb=0.3, periodic=False,
                                            codes={(0, 0): 10101, (0, 1): 10101, (1, 0): 10102, (1, 1): 10102}),
    # advection: inflow (b.n < 0) takes the exterior value, outflow the interior one
    "adv_upwind_box_8": lambda: M.mixed_advection_2d(8, seed=2, curved=True, periodic=False,
                                                     codes={(0, 0): 10041, (0, 1): 10041, (1, 0): 10001,
                                                            (1, 1): 10011}),
}


@pytest.mark.parametrize("name", sorted(BC_CASES))
@pytest.mark.parametrize("form", FORMS)
def test_boundaries_match_oracle(gpu_lib, name, form):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = BC_CASES[name]()
    ref = oracle.Oracle(prob)
    r_ref, mx_ref = ref.compute_rhs(prob.sol)
    s_ref = prob.sol.copy()
    for _ in range(2):
        s_ref, _, _ = ref.ssp_rk3_step(s_ref, prob.dt)
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx = sim.compute_rhs()
        r = sim.rhs
        sim.ssp_rk3_steps(prob.dt, 2)
        s = sim.sol_coef
    assert rel_err(r, r_ref) <= TOL
    assert abs(mx - mx_ref) <= TOL * mx_ref
    assert rel_err(s, s_ref) <= TOL


def test_boundaries_keep_the_free_stream(gpu_lib):
    from dpgsolver_gb300.solver import BatchSimulation
    for name in ("hex_roe_wall_riemann_4", "quad_roe_box_8"):
        prob = BC_CASES[name]()
        d = prob.d
        vel = 0.5 * np.sqrt(P.GAMMA) * np.array([1.0, 0.5, 0.25][:d]) / np.linalg.norm([1.0, 0.5, 0.25][:d])
        vel[1] = 0.0     # no flow through the slip walls (y = const)
        U = P.primitive_to_conserved(d, np.ones(1), vel[:, None], np.ones(1))[:, 0]
        s = np.concatenate([np.repeat(U, n) for n in prob.n_vs])
        prob.bc_state[:] = U
        with BatchSimulation(prob) as sim:
            sim.upload_state(s)
            assert sim.compute_rhs() < 1e-11


def test_ill_conditioned_case_within_rounding_noise(gpu_lib):
    """With small volumes and a small perturbation of the free stream, the residual is a small difference of
    large flux terms: h = 0.1 and 5 % perturbations make max|R| about 30 p^2 times smaller than the terms. Rounding
    the oracle's own input to the nearest neighbouring doubles (+-1 ulp) then already moves its residual by about
    1.3e-12 normwise, so no FP64 implementation can agree with it to 1e-12 there. The GPU residual must stay
    within 4x that measured noise floor."""
    from dpgsolver_gb300.solver import BatchSimulation
    prob = M.mixed_euler(3, 10, seed=6)
    ref = oracle.Oracle(prob)
    r_ref, _ = ref.compute_rhs(prob.sol)
    rng = np.random.default_rng(0)
    noise = 0.0
    for _ in range(3):
        s2 = prob.sol * (1.0 + rng.choice([-1.0, 1.0], size=prob.sol.shape) * 2.0 ** -53)
        noise = max(noise, rel_err(ref.compute_rhs(s2)[0], r_ref))
    assert noise > TOL   # the case is below the fixed tolerance's reach
    with BatchSimulation(prob) as sim:
        for form in FORMS:
            sim.form = form
            sim.compute_rhs()
            assert rel_err(sim.rhs, r_ref) <= 4.0 * noise


def test_forms_and_tiles_agree_bitwise(gpu_lib):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES["hex_roe_mixed_10"]()
    out = []
    with BatchSimulation(prob) as sim:
        for form, tiles in [("plain", None), ("fused", None), ("branches", None), ("stage", None),
                            ("plain", [1, 3, 2, 1]), ("branches", [4, 9, 1, 2])]:
            sim.form = form
            if tiles:
                for g, e in enumerate(tiles):
                    sim.set_group_tile(g, e)
            sim.upload_state(prob.sol)
            sim.compute_rhs()
            r = sim.rhs
            sim.ssp_rk3_steps(prob.dt, 2, want_max=False)
            out.append((r, sim.sol_coef))
    for r, s in out[1:]:
        assert np.array_equal(r, out[0][0])
        assert np.array_equal(s, out[0][1])


def test_uniform_mesh_as_one_group_matches_uniform_context(gpu_lib):
    """A uniform DGProblem through the batched context gives the uniform context's residual."""
    from dpgsolver_gb300.solver import BatchSimulation, Simulation
    prob = P.euler_hex_3d(4, 3, num_flux=P.NUM_FLUX_ROE_PIKE)
    with Simulation(prob) as u:
        u.compute_rhs()
        r_u = u.rhs
        u.ssp_rk3_steps(prob.dt, 2, want_max=False)
        s_u = u.sol_coef
    with BatchSimulation(prob) as b:
        b.compute_rhs()
        r_b = b.rhs
        b.ssp_rk3_steps(prob.dt, 2, want_max=False)
        s_b = b.sol_coef
    assert rel_err(r_b, r_u) <= 1e-14
    assert rel_err(s_b, s_u) <= 1e-14


def test_state_permutation_round_trip(gpu_lib):
    """Upload permutes list order into group order and download back: the identity on any state."""
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES["hex_roe_p24_5"]()
    rng = np.random.default_rng(11)
    s = rng.standard_normal(prob.n_state)
    with BatchSimulation(prob) as sim:
        sim.upload_state(s)
        assert np.array_equal(sim.sol_coef, s)


def test_autotune_keeps_state_and_results(gpu_lib):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES["hex_roe_mixed_10"]()
    with BatchSimulation(prob) as sim:
        sim.compute_rhs()
        r0 = sim.rhs
        rep = sim.autotune(prob.dt, reps=2)
        assert "plain" in rep and "fused" in rep and "branches" in rep and "stage" in rep and "E=" in rep
        assert np.array_equal(sim.sol_coef, prob.sol)
        sim.compute_rhs()
        assert np.array_equal(sim.rhs, r0)


def test_launch_counts(gpu_lib):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES["hex_roe_mixed_4"]()
    n_groups = len(prob.groups)
    n_face_orders = len(np.unique(prob.face_q))
    with BatchSimulation(prob) as sim:
        sim.compute_rhs()
        per_stage = 2 * n_groups + n_face_orders
        assert sim.kernel_launches() == per_stage
        sim.ssp_rk3_steps(prob.dt, 2)
        n1 = sim.kernel_launches()
        assert n1 == per_stage + n_groups + 2 * 3 * per_stage     # + the per-group V u conversion
        sim.form = "fused"
        sim.ssp_rk3_steps(prob.dt, 1)
        assert sim.kernel_launches() == n1 + 9
        sim.form = "branches"
        sim.ssp_rk3_steps(prob.dt, 1)
        assert sim.kernel_launches() == n1 + 9 + 3 * per_stage


def test_positivity_correction_matches_oracle(gpu_lib):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = M.mixed_vortex_2d(6, num_flux=P.NUM_FLUX_LAX_FRIEDRICHS, seed=7)
    sol = prob.sol.copy()
    for v in (0, 7, 20):
        b = prob.block(sol, v)
        n = 1
        scale = 1e-14 / b[0, n]
        b[0, n] *= scale
        b[1, n] *= scale
        b[2, n] *= scale
    ref = oracle.Oracle(prob)
    s_ref, _, ncorr_ref = ref.ssp_rk3_step(sol, 1e-4)
    assert ncorr_ref > 0
    for form in FORMS:
        with BatchSimulation(prob) as sim:
            sim.form = form
            sim.upload_state(sol)
            sim.ssp_rk3_steps(1e-4, 1)
            s = sim.sol_coef
            ncorr = sim.positivity_corrections()
        assert ncorr == ncorr_ref
        assert rel_err(s, s_ref) <= 1e-10


# ---- mixed element types: HEX (TP kernels) with TET / WEDGE / PYR (dense-operator kernels) ------------------------

def _types_case(n, seed, flux=P.NUM_FLUX_ROE_PIKE):
    from dpgsolver_gb300.host import mixed_types as MT
    return MT.mixed_types_euler(n, seed=seed, num_flux=flux, perturb=0.3)


TYPE_CASES = {
    "types_roe_4": lambda: _types_case(4, 0),
    "types_lf_4": lambda: _types_case(4, 1, P.NUM_FLUX_LAX_FRIEDRICHS),
    "types_roe_6": lambda: _types_case(6, 2),
    # every volume curved (the cube mapped by SineDeform): per-node metric terms, per-volume M^-1 of the dense groups
    "types_roe_curved_4": lambda: MT.mixed_types_euler(4, seed=0, perturb=0.3, curved=0.03),
}


@pytest.mark.parametrize("name", sorted(TYPE_CASES))
@pytest.mark.parametrize("form", FORMS)
def test_mixed_types_residual_matches_oracle(gpu_lib, name, form):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = TYPE_CASES[name]()
    r_ref, mx_ref = oracle.Oracle(prob).compute_rhs(prob.sol)
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx = sim.compute_rhs()
        r = sim.rhs
    assert rel_err(r, r_ref) <= TOL
    assert abs(mx - mx_ref) <= TOL * mx_ref


@pytest.mark.parametrize("name", ["types_roe_4", "types_roe_curved_4"])
@pytest.mark.parametrize("form", FORMS)
def test_mixed_types_rk3_matches_oracle(gpu_lib, form, name):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = TYPE_CASES[name]()
    ref = oracle.Oracle(prob)
    s_ref = prob.sol.copy()
    for _ in range(3):
        s_ref, mx_ref, _ = ref.ssp_rk3_step(s_ref, prob.dt)
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx = sim.ssp_rk3_steps(prob.dt, 3)
        s = sim.sol_coef
    assert rel_err(s, s_ref) <= TOL
    assert abs(mx - mx_ref) <= 1e-10 * mx_ref


def test_mixed_types_forms_and_tiles_agree_bitwise(gpu_lib):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = TYPE_CASES["types_roe_6"]()
    out = []
    with BatchSimulation(prob) as sim:
        for form, halve in [("plain", False), ("fused", False), ("branches", False), ("stage", False),
                            ("plain", True)]:
            sim.form = form
            if halve:
                for g in range(len(prob.groups)):
                    sim.set_group_tile(g, 1)
            sim.upload_state(prob.sol)
            sim.compute_rhs()
            r = sim.rhs
            sim.ssp_rk3_steps(prob.dt, 2, want_max=False)
            out.append((r, sim.sol_coef))
        rep = sim.autotune(prob.dt, reps=1)
        assert "dense group" in rep
    for r, s in out[1:]:
        assert np.array_equal(r, out[0][0])
        assert np.array_equal(s, out[0][1])


def test_wedge_factorised_equals_dense(gpu_lib):
    """The sum-factorised WEDGE volume term (TRI x LINE factors) gives the dense per-volume products' residual."""
    from dpgsolver_gb300.solver import BatchSimulation
    prob = TYPE_CASES["types_roe_6"]()
    r_ref, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    out = []
    for fac in (True, False):
        with BatchSimulation(prob, factorised=fac) as sim:
            sim.compute_rhs()
            out.append(sim.rhs)
    assert rel_err(out[0], r_ref) <= TOL
    assert rel_err(out[1], r_ref) <= TOL
    assert rel_err(out[0], out[1]) <= 1e-13


# ---- argument checking of dgpu_batch_create_groups (host-side validation, before any kernel) ---------------------

def _create_error(prob, **kw):
    from dpgsolver_gb300.solver import BatchSimulation, DGPUError
    with pytest.raises(DGPUError) as ei:
        BatchSimulation(prob, **kw)
    return ei.value


def test_one_curved_dense_volume_gets_its_own_mass_matrix(gpu_lib):
    """A single non-affine volume (J changed at one node) in an otherwise affine dense group: its group switches to
    per-volume M^-1 (formed on the device at creation), and the residual still matches the oracle's, which inverts
    that volume's M = cv0^T diag(w J) cv0 on its own."""
    from dpgsolver_gb300.solver import BatchSimulation
    prob = TYPE_CASES["types_roe_4"]()
    flat = prob.flat

    def bent():
        fl = flat()
        v = int(prob.group_vols[[getattr(o, "dense", False) for o in prob.groups].index(True)][0])
        n_vc = np.array([prob.groups[g].n_vc for g in prob.vol_group])
        off = int(np.sum(n_vc[:v]))
        fl["jacobian_det_vc"] = fl["jacobian_det_vc"].copy()
        fl["jacobian_det_vc"][off + 1] *= 1.01
        return fl
    prob.flat = bent
    r_ref, mx_ref = oracle.Oracle(prob).compute_rhs(prob.sol)
    with BatchSimulation(prob) as sim:
        mx = sim.compute_rhs()
        r = sim.rhs
    assert rel_err(r, r_ref) <= TOL
    assert abs(mx - mx_ref) <= TOL * mx_ref


def test_create_rejects_bad_orientation(gpu_lib):
    prob = TYPE_CASES["types_roe_4"]()
    flat = prob.flat

    def bad():
        fl = flat()
        fo = fl["face_ord"].copy()
        hexes = np.nonzero(np.array([not getattr(prob.groups[g], "dense", False) for g in prob.vol_group]))[0]
        f = int(np.nonzero(np.isin(prob.mesh.face_vol[:, 0], hexes))[0][0])
        fo[f, 0] = 3                       # a HEX side must see its face unpermuted
        fl["face_ord"] = fo
        return fl
    prob.flat = bad
    e = _create_error(prob)
    assert e.status == 2 and "face_ord 0" in str(e)
    prob.flat = flat

    def out_of_range():
        fl = flat()
        fo = fl["face_ord"].copy()
        dense = np.nonzero(np.array([getattr(prob.groups[g], "dense", False) for g in prob.vol_group]))[0]
        f = int(np.nonzero(np.isin(prob.mesh.face_vol[:, 1], dense))[0][0])
        fo[f, 1] = 9
        fl["face_ord"] = fo
        return fl
    prob.flat = out_of_range
    e = _create_error(prob)
    assert e.status == 1 and "face_ord" in str(e)


def test_create_rejects_wedge_factors_that_do_not_match(gpu_lib):
    prob = TYPE_CASES["types_roe_4"]()
    from dpgsolver_gb300.host.element import WEDGE
    g = [getattr(o, "e_type", None) for o in prob.groups].index(WEDGE)
    ops = prob.groups[g]
    good = ops.prism_factors

    def scaled():
        t0, t1, l0, l1 = good()
        return t0 * 1.001, t1, l0, l1
    ops.prism_factors = scaled
    e = _create_error(prob)
    assert e.status == 1 and "WEDGE factors" in str(e)
    ops.prism_factors = good


# ---- 2D: QUAD and TRI volumes (dense TRI groups, LINE faces in two orientations) -------------------------------
TRI_CASES = {
    "tri_quad_roe_6": lambda: MT.mixed_tri_quad_euler(6, seed=1),
    "tri_quad_lf_p13_8": lambda: MT.mixed_tri_quad_euler(8, seed=2, p_set=(1, 3),
                                                         num_flux=P.NUM_FLUX_LAX_FRIEDRICHS),
    "tri_only_roe_5": lambda: MT.mixed_tri_quad_euler(5, seed=3, p_tri=1.0),
    "tri_quad_curved_roe_6": lambda: MT.mixed_tri_quad_euler(6, seed=1, curved=0.03),
}


@pytest.mark.parametrize("name", sorted(TRI_CASES))
@pytest.mark.parametrize("form", FORMS)
def test_tri_quad_matches_oracle(gpu_lib, name, form):
    from dpgsolver_gb300.solver import BatchSimulation
    prob = TRI_CASES[name]()
    ref = oracle.Oracle(prob)
    r_ref, mx_ref = ref.compute_rhs(prob.sol)
    s_ref = prob.sol.copy()
    for _ in range(2):
        s_ref, _, _ = ref.ssp_rk3_step(s_ref, prob.dt)
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx = sim.compute_rhs()
        r = sim.rhs
        sim.ssp_rk3_steps(prob.dt, 2)
        s = sim.sol_coef
    assert rel_err(r, r_ref) <= TOL
    assert abs(mx - mx_ref) <= TOL * mx_ref
    assert rel_err(s, s_ref) <= TOL


@pytest.mark.parametrize("make", [lambda: MT.mixed_types_euler(4, seed=0, perturb=0.9),
                                  lambda: MT.mixed_tri_quad_euler(5, seed=4, perturb=0.97)])
def test_dense_positivity_matches_oracle(gpu_lib, make):
    """enforce_positivity_highorder on TRI/TET/WEDGE/PYR groups (their Bezier maps, simplex.bezier_basis): strong
    density and pressure dips trigger corrections; two RK steps in every form against the oracle, the same number
    of corrected volume-stages, at 1e-10 as the TP limiter's test (correct_coef's blend amplifies rounding)."""
    from dpgsolver_gb300.solver import BatchSimulation
    prob = make()
    prob.positivity = True
    ref = oracle.Oracle(prob)
    s_ref, ncorr_ref = prob.sol.copy(), 0
    for _ in range(2):
        s_ref, _, k = ref.ssp_rk3_step(s_ref, prob.dt)
        ncorr_ref += k
    assert ncorr_ref > 0
    for form in FORMS:
        with BatchSimulation(prob) as sim:
            sim.form = form
            sim.ssp_rk3_steps(prob.dt, 2)
            s = sim.sol_coef
            ncorr = sim.positivity_corrections()
        assert ncorr == ncorr_ref, form
        assert rel_err(s, s_ref) <= 1e-10, form


# ---- the reference's face interface: nc_fc instead of a canonical face-node order ------------------------------

@pytest.mark.parametrize("d,n", [(2, 6), (3, 3)])
@pytest.mark.parametrize("form", FORMS)
def test_rotated_frames_take_nc_fc(gpu_lib, tmp_path, d, n, form):
    """A mixed-order QUAD/HEX mesh read from a gmsh file whose volumes have random local frames: neighbours see their
    common face in different orientations, and the caller passes the reference's right-trace permutation nc_fc
    (get_operator__nc_fc_T) per face. Residual and RK steps against the oracle, and max |R| as on the same mesh with
    aligned frames."""
    from dpgsolver_gb300.host import gmsh as G
    from dpgsolver_gb300.solver import BatchSimulation
    path = str(tmp_path / f"box{d}.msh")
    G.write_box_msh(path, d, n, 0.0, 1.0, periodic=True, rotate_seed=3)
    prob = M.mixed_euler(d, n, seed=1, mesh=G.GmshTPMesh(G.GmshMesh(path, d)))
    ident = np.concatenate([np.arange(k) for k in np.diff(prob.face_off)])
    assert np.any(prob.nc_fc() != ident)
    ref = oracle.Oracle(prob)
    r_ref, mx_ref = ref.compute_rhs(prob.sol)
    s_ref = prob.sol.copy()
    for _ in range(2):
        s_ref, _, _ = ref.ssp_rk3_step(s_ref, prob.dt)
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx = sim.compute_rhs()
        r = sim.rhs
        sim.ssp_rk3_steps(prob.dt, 2)
        s = sim.sol_coef
    assert rel_err(r, r_ref) <= TOL
    assert abs(mx - mx_ref) <= TOL * mx_ref
    assert rel_err(s, s_ref) <= TOL
    aligned = M.mixed_euler(d, n, seed=1)
    with BatchSimulation(aligned) as sim:
        assert abs(sim.compute_rhs() - mx) <= 1e-12 * mx


def _reference_layout(prob):
    """The mixed-type mesh as the reference's face interface describes it: every side's face operators in its own
    face-node order (orientation 0), the face's data in side 0's own order, and nc_fc, the right-trace gather
    permutation, instead of the canonical order that orientation-specific operators produce."""
    fl0 = prob.flat()
    mesh = prob.mesh
    fo = np.asarray(fl0["face_ord"]).copy()
    nc = np.asarray(fl0["nc_fc"], dtype=np.int32).copy()
    d = prob.d
    nrm = np.asarray(fl0["normals_fc"]).reshape(-1, d).copy()
    jf = np.asarray(fl0["jacobian_det_fc"]).copy()

    def canon(f, s):   # own face node j -> canonical node
        v = int(mesh.face_vol[f, s])
        ops = prob.groups[prob.vol_group[v]]
        nf = int(prob.face_off[f + 1] - prob.face_off[f])
        if not getattr(ops, "dense", False) or fo[f, s] == 0:
            return np.arange(nf)
        lf, qf = int(mesh.face_lf[f, s]), int(prob.face_q[f])
        own, can = ops.face_points(lf, 0, qf), ops.face_points(lf, int(fo[f, s]), qf)
        return np.array([int(np.argmin(np.sum((can - x) ** 2, axis=1))) for x in own])
    for f in range(mesh.n_faces):
        a, b = int(prob.face_off[f]), int(prob.face_off[f + 1])
        c0 = canon(f, 0)
        nrm[a:b] = nrm[a:b][c0]
        jf[a:b] = jf[a:b][c0]
        if mesh.face_vol[f, 1] >= 0:
            c1 = canon(f, 1)
            inv1 = np.empty_like(c1)
            inv1[c1] = np.arange(len(c1))
            nc[a:b] = inv1[c0]
        fo[f] = 0
    flat = prob.flat

    def new_flat():
        fl = flat()
        fl.update(face_ord=fo, nc_fc=nc, normals_fc=nrm.ravel(), jacobian_det_fc=jf)
        return fl
    prob.flat = new_flat
    return prob


@pytest.mark.parametrize("form", FORMS)
def test_dense_faces_in_the_reference_layout(gpu_lib, form):
    """TET/WEDGE/PYR sides given their own-order face operators and nc_fc (as the reference's shim would pass them)
    instead of orientation-specific operators: the same residual as the canonical layout, and the oracle's."""
    from dpgsolver_gb300.solver import BatchSimulation
    prob = TYPE_CASES["types_roe_4"]()
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx_can = sim.compute_rhs()
        r_can = sim.rhs
    prob = _reference_layout(prob)
    ident = np.concatenate([np.arange(k) for k in np.diff(prob.face_off)])
    assert np.any(prob.flat()["nc_fc"] != ident) and not np.any(prob.flat()["face_ord"])
    r_ref, mx_ref = oracle.Oracle(prob).compute_rhs(prob.sol)
    with BatchSimulation(prob) as sim:
        sim.form = form
        mx = sim.compute_rhs()
        r = sim.rhs
        sim.ssp_rk3_steps(prob.dt, 1)
    assert rel_err(r, r_ref) <= TOL
    assert rel_err(r, r_can) <= TOL
    assert abs(mx - mx_can) <= TOL * mx_can


def test_stage_barrier_wait_is_bounded_and_the_context_recovers(gpu_lib):
    """The "stage" form's grid barriers wait a bounded time: with a bound of 1 ns the waits run out (most CTAs have
    no tile of this small mesh and wait for the others), the stage kernel ends and the call returns DGPU_ERR_CUDA;
    with the default bound the same context then computes the oracle's residual. Nothing waits without a bound."""
    from dpgsolver_gb300._lib import DGPUError
    from dpgsolver_gb300.solver import BatchSimulation
    prob = CASES["hex_roe_mixed_4"]()
    r_ref, _ = oracle.Oracle(prob).compute_rhs(prob.sol)
    with BatchSimulation(prob) as sim:
        sim.form = "stage"
        sim.set_barrier_timeout(1e-9)
        with pytest.raises(DGPUError) as e:
            sim.compute_rhs()
        assert e.value.status == 3 and "barrier" in str(e.value)
        sim.set_barrier_timeout(2.0)
        sim.upload_state(prob.sol)
        sim.compute_rhs()
        assert rel_err(sim.rhs, r_ref) <= TOL
