"""The reference's own 2D explicit-DG code, compiled into ``oracle/_ref`` by ``oracle/ref/Makefile`` (TEST
INFRASTRUCTURE ONLY: it pins the oracle and the kernels to residuals the reference itself computes; nothing on the
product path imports it).

``build(ref_dir)`` compiles the reference's ``src/`` tree where it lies, with the stand-ins of ``oracle/ref/shim``;
``run_case(...)`` writes a control file, the test case's ``test_case.data`` / ``solution.data`` and a gmsh 2.2 mesh
under ``oracle/_ref/run/input`` (the input directory compiled into the build), runs ``dpg_ref_harness`` and reads
back what it wrote: the volume and face lists in the reference's own order with their geometry, and, given a state,
``compute_rhs`` and the SSP-RK3 steps of ``time_step_ssp_rk_33``.

The reference cannot travel to the GPU machine (it is built here, for this host, from the reference's sources), so the
GPU tests use fixtures generated from it by ``tests/golden/make_ref_golden.py``.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(_HERE, "_ref")
HARNESS = os.path.join(REF_OUT, "dpg_ref_harness")
RUN_DIR = os.path.join(REF_OUT, "run")
INPUT_DIR = os.path.join(RUN_DIR, "input")


def available() -> bool:
    return os.path.exists(HARNESS)


def build(ref_dir: str, jobs: int | None = None) -> str:
    """Compile oracle/_ref/dpg_ref_harness from the reference checkout at ref_dir."""
    jobs = jobs or max(1, os.cpu_count() or 1)
    subprocess.run(["make", "-s", "-C", os.path.join(_HERE, "ref"), f"REF={ref_dir}", f"-j{jobs}"], check=True)
    return HARNESS


_CTRL = """pde_name  {pde_name}
pde_spec  {pde_spec}

geom_name {geom_name}
geom_spec {geom_spec}

dimension 2

mesh_generator   n-cube/2d.geo
mesh_format      gmsh
mesh_domain      {domain}
mesh_type        quad
mesh_level       0 0
mesh_path        {mesh}

interp_tp  GLL
interp_si  AO
interp_pyr GLL

basis_geom  bezier
basis_sol   lagrange

geom_representation  isoparametric
geom_blending_tp     gordon_hall
geom_blending_si     szabo_babuska_gen

p_ref    {p} {p_max}

fe_method 1
"""

_TEST_CASE = """solver_proc   explicit
solver_type_e ssp_rk_33

num_flux_1st {num_flux}
{extra}
time_step  {dt!r}
time_final {t_final!r}

display_progress 0
"""

# The reference's own spelling of the numerical fluxes in test_case.data (test_case_T.c:277 converts them).
NUM_FLUX_NAMES = {11: "upwind", 31: "Roe-Pike", 32: "Lax-Friedrichs"}


def _write(path: str, text: str) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as fh:
        fh.write(text)


def _read_bin(path: str) -> np.ndarray:
    return np.fromfile(path, dtype=np.float64)


def write_tri_quad_msh(path: str, mesh) -> None:
    """A MixedTriQuadMesh (unit square, QUAD and TRI cells) as a gmsh 2.2 file the way the reference's meshes come: one
    node per grid point of the (n+1)^2 grid, the boundary lines, then the volumes in the mesh's own order (TRI: gmsh
    type 2, QUAD: type 3 with gmsh's counter-clockwise vertex order). A periodic mesh gets the periodic codes
    10051/10052 (x) and 10053/10054 (y) and a $Periodic section, otherwise slip walls (10102) on every side."""
    n = mesh.n
    node = lambda i, j: i + (n + 1) * j + 1
    lines = []
    periodic = getattr(mesh, "periodic", True)
    sides = ((10053, 1002), (10054, 1003), (10051, 1000), (10052, 1001)) if periodic else \
        ((10102, 1002), (10102, 1003), (10102, 1000), (10102, 1001))   # slip walls
    for k, (code, ent) in enumerate(sides):
        for c in range(n):
            if k == 0:
                a, b = node(c, 0), node(c + 1, 0)
            elif k == 1:
                a, b = node(c, n), node(c + 1, n)
            elif k == 2:
                a, b = node(0, c), node(0, c + 1)
            else:
                a, b = node(n, c), node(n, c + 1)
            lines.append(f"1 2 {code} {ent} {a} {b}")
    for v in range(mesh.n_volumes):
        ij = np.rint(np.asarray(mesh.X[v]) / mesh.h).astype(int)
        ids = [node(i, j) for i, j in ij]
        if len(ids) == 3:
            lines.append("2 2 9401 4001 " + " ".join(map(str, ids)))
        else:   # TP corner order (0,0) (1,0) (0,1) (1,1) -> gmsh (0,0) (1,0) (1,1) (0,1)
            lines.append("3 2 9401 4001 " + " ".join(map(str, [ids[0], ids[1], ids[3], ids[2]])))
    with open(path, "w") as fh:
        fh.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % ((n + 1) ** 2))
        for j in range(n + 1):
            for i in range(n + 1):
                fh.write("%d %.17g %.17g 0\n" % (node(i, j), i * mesh.h, j * mesh.h))
        fh.write("$EndNodes\n$Elements\n%d\n" % len(lines))
        for e, ln in enumerate(lines):
            fh.write(f"{e + 1} {ln}\n")
        fh.write("$EndElements\n")
        if periodic:
            fh.write("$Periodic\n2\n1 1001 1000\n0\n1 1003 1002\n0\n$EndPeriodic\n")


def run_case(name: str, pde: str, n: int, p: int, lo: float, hi: float, num_flux: int, state_fn=None,
             steps: int = 0, dt: float = 0.0, map_amplitude: float = 0.0, b_adv=(1.0, 0.5), mesh_writer=None,
             states_fn=None, pde_spec: str | None = None, ns: dict | None = None, bc_data=None,
             mach: float = 0.4, adapt_p=None, p_max: int | None = None) -> dict:
    """Set up a periodic n x n mesh of [lo, hi]^2 at order p in the reference and run it.

    pde: "advection" (upwind, b_adv) or "euler". map_amplitude > 0 makes the domain parametric with the map
    x, y += A sin(2 pi x / (hi - lo)) sin(2 pi y / (hi - lo)). The mesh is the QUAD box of write_box_msh unless
    mesh_writer(path) writes another. state_fn(xyz_vs) -> (n_vs, n_var) gives the initial nodal state of a volume from
    its solution-node coordinates (Lagrange coefficients are nodal values); states_fn(geometry) -> one such array per
    volume is the alternative that sees the whole geometry dump. With either, the reference's compute_rhs and
    ``steps`` SSP-RK3 steps of size dt are run. pde_spec overrides the test case (advection: "steady/free_stream",
    no source; "steady/default", the source of solution_advection_default_T.c). pde "navier_stokes" runs the
    reference's steady/taylor_couette case on the parametric mesh of mesh_writer with the constants of ns (mu, Pr,
    r_s, omega, p_b, t_b, rho_b, E_b and dTdn; dTdn != 0 makes the outer wall diabatic), BR2 for the viscous terms.
    Euler with pde_spec "steady/free_stream" takes bc_data = (p_back, t_total, p_total, r_s) for its back-pressure
    and total T/p faces; "steady/supersonic_vortex" runs the supersonic vortex on the parametric quarter annulus.
    adapt_p: [(x, y, p), ...] adapts the orders around those vertices after set-up (the harness's --adapt-p); every
    volume starts at p and may move within [p, p_max] (the control file's p_ref range).
    """
    from dpgsolver_gb300.host.gmsh import write_box_msh

    if not available():
        raise RuntimeError("oracle/_ref is not built")
    ctrl_name = f"TEST_ref_{name}"
    case_dir = os.path.join(RUN_DIR, name)
    os.makedirs(case_dir, exist_ok=True)
    mesh = os.path.join(case_dir, "mesh.msh")
    if mesh_writer is None:
        write_box_msh(mesh, 2, n, lo=lo, hi=hi, periodic=True)
    else:
        mesh_writer(mesh)
    geom_name, geom_spec, extra = "n-cube", "NONE", ""
    domain = "parametric" if map_amplitude else "straight"
    if pde == "advection":
        pde_spec = pde_spec or "steady/free_stream"
        solution = f"advection_type constant\nb_adv   {b_adv[0]!r} {b_adv[1]!r} 0.0\n"
    elif pde == "euler" and pde_spec == "steady/free_stream":
        # the stream of the subsonic duct; the back-pressure and total T/p faces read their data here too
        p_back, t_total, p_total, r_s = bc_data
        solution = (f"density   1.0\npressure  1.0\nmach      {mach!r}\ntheta_deg 0.0\n\nboundary_perturb_type none\n\n"
                    f"p_back  {p_back!r}\nt_total {t_total!r}\np_total {p_total!r}\nr_s     {r_s!r}\n")
    elif pde == "euler" and pde_spec == "steady/supersonic_vortex":
        geom_name, domain = "n-cylinder_hollow_section", "parametric"
        solution = "m_i   2.25\nrho_i 1.0\n"
    elif pde == "euler":
        pde_spec = pde_spec or "periodic/periodic_vortex"
        solution = ("r_v   0.165\ntheta 0.7853981633974483\nV_inf 0.5916079783099616\np_inf 1.0\nt_inf 1.0\n"
                    "Rg    1.0\n\np_frac 0.05\n")
    elif pde == "navier_stokes":
        pde_spec = pde_spec or "steady/taylor_couette"
        geom_name, domain, extra = "n-cylinder_hollow", "parametric", "num_flux_2nd BR2_stable\n"
        geom_spec = ("diabatic_o" if ns["dTdn"] != 0.0 else "adiabatic_o") + "/geom_ar_1"
        flux_type = "constant" if ns["dTdn"] != 0.0 else "constant_zero"
        visc = "sutherland" if ns.get("viscosity") == 102 else "constant"
        solution = (f"Pr  {ns['Pr']!r}\nr_s {ns['r_s']!r}\n\nviscosity_type {visc}\nmu {ns['mu']!r}\n\n"
                    f"diabatic_flux_type {flux_type}\ndTdn {ns['dTdn']!r}\n\nno_slip_type rotating\n"
                    f"omega {ns['omega']!r}\n\nno_slip_all_type density_energy\np_b {ns['p_b']!r}\n"
                    f"t_b {ns['t_b']!r}\n\nrho_b {ns['rho_b']!r}\nE_b {ns['E_b']!r}\n")
    else:
        raise ValueError(pde)
    _write(os.path.join(INPUT_DIR, "testing", "control_files", ctrl_name + ".ctrl"),
           _CTRL.format(pde_name=pde, pde_spec=pde_spec, geom_name=geom_name, geom_spec=geom_spec, domain=domain, mesh=mesh, p=p,
                       p_max=p if p_max is None else p_max))
    data_dir = os.path.join(INPUT_DIR, "input_files", pde, pde_spec)
    _write(os.path.join(data_dir, "test_case.data"),
           _TEST_CASE.format(num_flux=NUM_FLUX_NAMES[num_flux], extra=extra, dt=float(dt or 1e-3),
                             t_final=float((dt or 1e-3) * max(steps, 1))))
    _write(os.path.join(data_dir, "solution.data"), solution)
    if pde == "navier_stokes":   # the annulus radii the Taylor-Couette solution functions read
        _write(os.path.join(data_dir, "geometry_parameters.geo"), "r_i = 0.5;\nr_o = 1.0;\n")
    if pde_spec == "steady/supersonic_vortex":
        _write(os.path.join(data_dir, "geometry_parameters.geo"), "r_i = 1.0;\nr_o = 1.384;\n")

    args = [HARNESS, ctrl_name, case_dir]
    if pde_spec in ("steady/supersonic_vortex", "steady/default", "steady/free_stream") and mesh_writer is not None:
        args.append("--keep-sol")   # boundary faces that read the test case's solution
    if map_amplitude:
        args += ["--map", repr(float(map_amplitude)), repr(float(hi - lo))]
    if adapt_p:
        path = os.path.join(case_dir, "adapt.txt")
        with open(path, "w") as fh:
            for x, y, q in adapt_p:
                fh.write(f"{float(x)!r} {float(y)!r} {int(q)}\n")
        args += ["--adapt-p", path]
    subprocess.run(args, check=True, cwd=case_dir, stdout=subprocess.DEVNULL)
    out = _read_outputs(case_dir)
    if state_fn is not None or states_fn is not None:
        blocks = states_fn(out) if states_fn is not None else [state_fn(x) for x in out["xyz_vs"]]
        sol = np.concatenate([np.asarray(b, dtype=np.float64).reshape(x.shape[0], -1).T.ravel()
                              for b, x in zip(blocks, out["xyz_vs"])])
        sol.tofile(os.path.join(case_dir, "sol_in.bin"))
        args += ["--state", os.path.join(case_dir, "sol_in.bin")]
        if steps:
            args += ["--steps", str(int(steps)), "--dt", repr(float(dt))]
        subprocess.run(args, check=True, cwd=case_dir, stdout=subprocess.DEVNULL)
        out.update(_read_outputs(case_dir))
        out["sol_in"] = sol
        n_var = sol.size // sum(x.shape[0] for x in out["xyz_vs"])
        out["n_var"] = n_var
        out["rhs"] = _read_bin(os.path.join(case_dir, "rhs.bin"))
        mx = np.loadtxt(os.path.join(case_dir, "max_rhs.txt"), ndmin=1)
        out["max_rhs"] = float(mx[0])
        if steps:
            out["max_rhs_steps"] = mx[1:]
            out["sol_steps"] = _read_bin(os.path.join(case_dir, "sol_steps.bin"))
    return out


def _read_outputs(case_dir: str) -> dict:
    vols = np.loadtxt(os.path.join(case_dir, "volumes.txt"), dtype=np.int64, ndmin=2)
    faces = np.loadtxt(os.path.join(case_dir, "faces.txt"), dtype=np.int64, ndmin=2)
    d = 2
    n_vs, n_vc, n_ve = vols[:, 4], vols[:, 5], vols[:, 6]

    def split(arr, sizes):
        return np.split(arr, np.cumsum(sizes)[:-1])

    def cols(blocks, sizes, k):
        # column-major (n, k) blocks -> list of (n, k) arrays
        return [b.reshape(k, n).T for b, n in zip(blocks, sizes)]

    # Volume::xyz_ve is row-major ('R'), like normals_fc
    xyz_ve = [b.reshape(nn, d) for b, nn in zip(split(_read_bin(os.path.join(case_dir, "xyz_ve.bin")), n_ve * d), n_ve)]
    xyz_vs = cols(split(_read_bin(os.path.join(case_dir, "xyz_vs.bin")), n_vs * d), n_vs, d)
    met = split(_read_bin(os.path.join(case_dir, "metrics_vc.bin")), n_vc * d * d)
    # metrics_vc (n_vc, d, d) column-major: entry (n, i, j) at n + n_vc (i + d j)
    metrics = [m.reshape(d, d, nc).transpose(2, 1, 0) for m, nc in zip(met, n_vc)]
    jac = split(_read_bin(os.path.join(case_dir, "jacobian_det_vc.bin")), n_vc)
    n_fc = faces[:, 3]
    # normals_fc is the reference's one row-major ('R') face multiarray (face_solver_T.h:56)
    normals = [b.reshape(nf, d) for b, nf in zip(split(_read_bin(os.path.join(case_dir, "normals_fc.bin")), n_fc * d),
                                                  n_fc)]
    jac_f = split(_read_bin(os.path.join(case_dir, "jacobian_det_fc.bin")), n_fc)
    xyz_fc = cols(split(_read_bin(os.path.join(case_dir, "xyz_fc.bin")), n_fc * d), n_fc, d)
    return dict(volumes=vols, faces=faces, xyz_ve=xyz_ve, xyz_vs=xyz_vs, metrics_vc=metrics, jacobian_det_vc=jac,
                normals_fc=normals, jacobian_det_fc=jac_f, xyz_fc=xyz_fc)


# ------------------------------------------------------------------------------------------------------------------
# The parity cases run through the reference, and their counterparts built by the repo's own host set-up.

def _advection_state(x):
    return np.sin(np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1])


def _advection_default_state(x):
    from dpgsolver_gb300.host.problem import SOURCE_A, SOURCE_M
    return np.sin(SOURCE_M * x[:, 0] + SOURCE_A) * np.sin(SOURCE_M * x[:, 1] + SOURCE_A)


def _sv_state(x):
    from dpgsolver_gb300.host.problem import supersonic_vortex_state
    X, Y = x[:, 0], x[:, 1]
    R, TH = np.sqrt(X * X + Y * Y), np.arctan2(Y, X)
    return (np.asarray(supersonic_vortex_state(X, Y)) *
            (1.0 + 0.05 * np.sin(4.0 * TH) * np.sin(np.pi * (R - 1.0) / 0.384))[None]).T


def _duct_state(x):
    from dpgsolver_gb300.host.problem import subsonic_duct_state
    return np.asarray(subsonic_duct_state(x, 2, 0.4, 0.02, 0)).T


def _sduct_state(x):
    from dpgsolver_gb300.host.problem import subsonic_duct_state
    return np.asarray(subsonic_duct_state(x, 2, 1.5, 0.02, 0)).T


def _tc_state(x, diabatic):
    from dpgsolver_gb300.host.problem import taylor_couette_state
    X, Y = x[:, 0], x[:, 1]
    U = taylor_couette_state(X, Y, 0.5, 1.0, 1.0, _TC_MU, 0.72, 1.0, 1.0, 1.0, 1.0 if diabatic else 0.0)
    R, TH = np.sqrt(X * X + Y * Y), np.arctan2(Y, X)
    return (np.asarray(U) * (1.0 + 0.2 * np.sin(3.0 * TH) * np.sin(np.pi * (R - 0.5) / 0.5))[None]).T


def _pos_dip(x):
    """The near-vacuum dip of the positivity case: every conserved variable scaled by
    1 - (1 - 1e-6) exp(-|x - (5, 5)|^2 / 0.09) (velocity and temperature unchanged)."""
    return 1.0 - (1.0 - 1e-6) * np.exp(-((x[:, 0] - 5.0) ** 2 + (x[:, 1] - 5.0) ** 2) / 0.09)


def _vortex_state(x):
    from dpgsolver_gb300.host.problem import isentropic_vortex, primitive_to_conserved
    rho, u, v, pr = isentropic_vortex(x, 5.0, 5.0, 5.0)
    return np.asarray(primitive_to_conserved(2, rho, np.stack([u, v]), pr)).T


# name -> (pde, n, p, numerical flux, RK steps). "c1" is the linear-advection configuration at its stated size
# (QUAD 16^2 on [-1,1]^2, p = 2, b = (1, 0.5), upwind, u0 = sin(pi x) sin(pi y), dt = 0.1 h / |b|, 100 steps);
# the "c2*" cases are the curved isentropic-vortex configuration (QUAD on [0,10]^2 mapped by
# 0.05 sin(pi x/5) sin(pi y/5), vortex strength 5 at (5,5) on (1,1,1,1)) on smaller meshes and other fluxes and
# orders ("c2_pos_n8": the vortex with a near-vacuum dip at its centre, density and energy scaled down to 1e-6 there,
# which makes enforce_positivity_highorder correct volumes in every step: 32 corrections in its 5 steps; the limiter's
# blend amplifies rounding, so longer runs drift apart: 1.5e-13 after one step, 2.4e-13 after five, 6.6e-10 after
# twenty between the oracle and the reference); "c2" itself (64^2, p = 3, Roe) is run live by the CPU tests. "c1_source" is the reference's steady
# advection case with a source term (steady/default: u = sin(2.15 x + 0.23) sin(2.15 y + 0.23), s = b . grad u) on
# a periodic QUAD 8^2 mesh of [-1,1]^2 mapped by 0.05 sin(pi x) sin(pi y), p = 3, upwind, 20 steps; "c1_source_bc"
# the same case on a 6^2 box with upwind boundaries (BC_UPWIND) on its four sides, whose exterior state is the test
# case's steady solution. "tc_*" are the
# reference's Navier-Stokes Taylor-Couette case (steady/taylor_couette, mu = 0.02, omega = 1) on its parametric square
# annulus with 2 x 2 volumes per block (16 volumes): rotating inner wall, adiabatic (p = 3) or diabatic (dTdn = 1,
# p = 2) outer wall; Roe-Pike (the only inviscid flux the reference's Navier-Stokes takes) and BR2, the state
# perturbed by 20 %, 10 steps ("tc_suth_n2": adiabatic, with Sutherland's law scaled by mu). "duct_*" are the subsonic duct on a straight 4^2 / 3^2 box of [0,10]^2 in the
# reference's free-stream case with its internal-flow boundaries (n-cube/2d.geo, GEOM_ADV_INTERNAL): total T/p inflow,
# back-pressure outflow, slip walls; Roe-Pike p = 3, Lax-Friedrichs p = 2, 10 steps. "sduct_n4": the same box at
# Mach 1.5 with supersonic inflow (the free stream outside) and outflow (GEOM_ADV_XL), Roe-Pike p = 3. "sv_*" are the reference's Euler supersonic vortex (steady/supersonic_vortex,
# m_i = 2.25) on its parametric quarter square annulus (3 x 3 and 2 x 2 volumes per block): Riemann faces with the
# exact solution outside, slip walls on both arcs; Roe-Pike p = 3 and Lax-Friedrichs p = 2, density perturbed by 5 %.
CASES = {
    "c1": ("advection", 16, 2, 11, 100),
    "c1_source": ("advection_default", 8, 3, 11, 20),
    "c1_source_bc": ("advection_default_bc", 6, 3, 11, 20),
    "tc_n2": ("navier_stokes_tc", 2, 3, 31, 10),
    "tc_suth_n2": ("navier_stokes_tc_sutherland", 2, 3, 31, 10),
    "duct_n4": ("euler_duct", 4, 3, 31, 10),
    "duct_lf_p2_n3": ("euler_duct", 3, 2, 32, 10),
    "sduct_n4": ("euler_sduct", 4, 3, 31, 10),
    "sv_n3": ("euler_sv", 3, 3, 31, 10),
    "sv_lf_p2_n2": ("euler_sv", 2, 2, 32, 10),
    "tc_diab_n2": ("navier_stokes_tc_diabatic", 2, 2, 31, 10),
    "c2_n8": ("euler", 8, 3, 31, 1000),
    "c2_lf_n8": ("euler", 8, 3, 32, 20),
    "c2_p1_n8": ("euler", 8, 1, 32, 20),
    "c2_p4_n4": ("euler", 4, 4, 31, 20),
    "c2_pos_n8": ("euler_pos", 8, 3, 31, 5),
    "c2": ("euler", 64, 3, 31, 10),
}


def host_problem(name: str):
    """The repo's own host set-up of a case (mesh, operators, geometry, state, dt)."""
    from dpgsolver_gb300.host import problem as P
    pde, n, p, flux, steps = CASES[name]
    if pde == "advection":
        return P.advection_2d(n, p)
    if pde == "advection_default":
        return P.advection_default_2d(n, p, n_steps=steps)
    if pde == "advection_default_bc":
        return P.advection_default_2d(n, p, n_steps=steps, periodic=False)
    if pde == "euler_duct":
        return P.euler_subsonic_duct(2, n, p, num_flux=flux, amplitude=0.0)
    if pde == "euler_sduct":
        return P.euler_supersonic_duct_2d(n, p, num_flux=flux)
    if pde == "euler_pos":
        prob = P.euler_vortex_2d(n=n, p=p, num_flux=flux)
        x = prob.solution_node_xyz()
        prob.sol = prob.sol * _pos_dip(x.reshape(-1, 2)).reshape(x.shape[:2])[:, None, :]
        return prob
    if pde == "euler_sv":
        return P.euler_supersonic_vortex(_case_mesh(name, lambda path: _sv_mesh(path, n)), p, num_flux=flux,
                                         perturb=0.05)
    if pde.startswith("navier_stokes_tc"):
        return P.ns_taylor_couette_parametric(_tc_mesh(name, n, pde.endswith("diabatic")), p, mu=_TC_MU,
                                              diabatic=pde.endswith("diabatic"), num_flux=flux, perturb=0.2,
                                              viscosity=P.VISCOSITY_SUTHERLAND if "sutherland" in pde
                                              else P.VISCOSITY_CONSTANT)
    return P.euler_vortex_2d(n=n, p=p, num_flux=flux)


_TC_MU = 0.02


def _case_mesh(name: str, writer) -> str:
    """A case's mesh file, written by writer(path) into the temporary directory."""
    import tempfile
    path = os.path.join(tempfile.gettempdir(), f"dpgsolver_gb300_{name}_{os.getpid()}.msh")
    writer(path)
    return path


def _tc_mesh(name: str, n: int, diabatic: bool) -> str:
    """The Taylor-Couette cases' square-annulus mesh (n x n volumes per block)."""
    from dpgsolver_gb300.host.gmsh import write_square_annulus_msh
    return _case_mesh(name, lambda path: write_square_annulus_msh(path, n, n, outer=20112 if diabatic else 20111))


def _sv_mesh(path: str, n: int) -> None:
    """The supersonic vortex cases' quarter square annulus (n x n volumes per block)."""
    from dpgsolver_gb300.host.gmsh import write_quarter_square_annulus_msh
    write_quarter_square_annulus_msh(path, n, n)


def run_named(name: str) -> dict:
    """Run a case through the reference with the host problem's dt; returns run_case's dictionary."""
    pde, n, p, flux, steps = CASES[name]
    prob = host_problem(name)
    if pde == "advection":
        return run_case(name, pde, n, p, -1.0, 1.0, flux, state_fn=_advection_state, steps=steps, dt=prob.dt)
    if pde == "advection_default_bc":   # upwind faces on the four sides, the steady solution outside
        from dpgsolver_gb300.host.gmsh import write_box_msh
        codes = {(k, s): 10041 for k in range(2) for s in range(2)}
        return run_case(name, "advection", n, p, -1.0, 1.0, flux, state_fn=_advection_default_state, steps=steps,
                        dt=prob.dt, map_amplitude=prob.meta["amplitude"], pde_spec="steady/default",
                        mesh_writer=lambda path: write_box_msh(path, 2, n, lo=-1.0, hi=1.0, periodic=False,
                                                               codes=codes))
    if pde == "advection_default":
        return run_case(name, "advection", n, p, -1.0, 1.0, flux, state_fn=_advection_default_state, steps=steps,
                        dt=prob.dt, map_amplitude=prob.meta["amplitude"], pde_spec="steady/default")
    if pde == "euler_pos":
        def pos_state(x):
            return _vortex_state(x) * _pos_dip(x)[:, None]
        return run_case(name, "euler", n, p, 0.0, 10.0, flux, state_fn=pos_state, steps=steps, dt=prob.dt,
                        map_amplitude=0.05)
    if pde == "euler_sduct":   # supersonic in/out faces (n-cube/2d.geo, GEOM_ADV_XL), slip walls
        from dpgsolver_gb300.host.gmsh import write_box_msh
        from dpgsolver_gb300.host.problem import subsonic_duct_state

        def sduct_state(x):
            return np.asarray(subsonic_duct_state(x, 2, 1.5, 0.02, 0)).T
        codes = {(0, 0): 10105, (0, 1): 10106, (1, 0): 10102, (1, 1): 10102}
        return run_case(name, "euler", n, p, 0.0, 10.0, flux, state_fn=sduct_state, steps=steps, dt=prob.dt,
                        mesh_writer=lambda path: write_box_msh(path, 2, n, lo=0.0, hi=10.0, periodic=False,
                                                               codes=codes),
                        pde_spec="steady/free_stream", bc_data=(0.0, 0.0, 0.0, 0.0), mach=1.5)
    if pde == "euler_duct":
        from dpgsolver_gb300.host.gmsh import write_box_msh
        from dpgsolver_gb300.host.problem import subsonic_duct_state

        def duct_state(x):
            return np.asarray(subsonic_duct_state(x, 2, 0.4, 0.02, 0)).T
        codes = {(0, 0): 10104, (0, 1): 10103, (1, 0): 10102, (1, 1): 10102}
        return run_case(name, "euler", n, p, 0.0, 10.0, flux, state_fn=duct_state, steps=steps, dt=prob.dt,
                        mesh_writer=lambda path: write_box_msh(path, 2, n, lo=0.0, hi=10.0, periodic=False,
                                                               codes=codes),
                        pde_spec="steady/free_stream", bc_data=prob.bc_data)
    if pde == "euler_sv":
        def sv_states(out):   # the host problem's state formula at the reference's solution nodes
            return [_sv_state(x) for x in out["xyz_vs"]]
        return run_case(name, "euler", n, p, 0.0, 1.0, flux, states_fn=sv_states, steps=steps, dt=prob.dt,
                        mesh_writer=lambda path: _sv_mesh(path, n), pde_spec="steady/supersonic_vortex")
    if pde.startswith("navier_stokes_tc"):
        from dpgsolver_gb300.host.gmsh import write_square_annulus_msh
        diabatic = pde.endswith("diabatic")
        ns = dict(prob.ns, omega=1.0, p_b=1.0, t_b=1.0, rho_b=1.0, E_b=1.0 / 0.4 + 0.5 * 0.5 ** 2)

        def states(out):   # the host problem's state formula at the reference's solution nodes
            return [_tc_state(x, diabatic) for x in out["xyz_vs"]]
        return run_case(name, "navier_stokes", n, p, 0.0, 1.0, flux, states_fn=states, steps=steps, dt=prob.dt,
                        mesh_writer=lambda path: write_square_annulus_msh(path, n, n,
                                                                          outer=20112 if diabatic else 20111),
                        ns=ns)
    return run_case(name, pde, n, p, 0.0, 10.0, flux, state_fn=_vortex_state, steps=steps, dt=prob.dt,
                    map_amplitude=0.05)


def to_arrays(out: dict) -> dict:
    """The reference's run in the host problem's layouts (what the golden fixtures store)."""
    nv = len(out["xyz_vs"])
    n_var = out.get("n_var", 1)
    res = dict(
        xyz_vs=np.stack(out["xyz_vs"]),
        metrics_vc=np.stack(out["metrics_vc"]),
        jacobian_det_vc=np.stack(out["jacobian_det_vc"]),
        normals_fc=np.stack(out["normals_fc"]),
        jacobian_det_fc=np.stack(out["jacobian_det_fc"]),
        face_vol=out["faces"][:, [4, 7]].astype(np.int32),
        face_lf=out["faces"][:, [5, 8]].astype(np.int32),
        face_ord=out["faces"][:, [6, 9]].astype(np.int32),
    )
    if "sol_in" in out:
        res.update(sol_in=out["sol_in"].reshape(nv, n_var, -1), rhs=out["rhs"].reshape(nv, n_var, -1),
                   max_rhs=np.float64(out["max_rhs"]))
    if "sol_steps" in out:
        res.update(sol_steps=out["sol_steps"].reshape(nv, n_var, -1), max_rhs_steps=out["max_rhs_steps"])
    return res


def with_reference_inputs(prob, ref: dict):
    """Give the host problem the reference's own geometry and initial state: what a caller packing the reference's
    Solver_Volume / Solver_Face lists would pass. Checks first that both list the same volumes (solution nodes within
    1e-12) and faces (volumes and local faces per side, identity face-node orders on interior faces) in the same
    order."""
    xyz = prob.solution_node_xyz()
    if np.abs(xyz - ref["xyz_vs"]).max() > _XYZ_TOL.get(prob.name, 1e-12):
        raise AssertionError("volume lists differ")
    interior = ref["face_vol"][:, 1] >= 0
    if not (np.array_equal(prob.mesh.face_vol, ref["face_vol"]) and np.array_equal(prob.mesh.face_lf, ref["face_lf"])
            and not np.any(ref["face_ord"][interior])):
        raise AssertionError("face lists differ")
    g = prob.geom
    g.metrics_vc = np.array(ref["metrics_vc"], dtype=np.float64)
    g.jacobian_det_vc = np.array(ref["jacobian_det_vc"], dtype=np.float64)
    g.normals_fc = np.array(ref["normals_fc"], dtype=np.float64)
    g.jacobian_det_fc = np.array(ref["jacobian_det_fc"], dtype=np.float64)
    if "sol_in" in ref:
        prob.sol = np.array(ref["sol_in"], dtype=np.float64)
    return prob


# ------------------------------------------------------------------------------------------------------------------
# Mixed-order meshes: the reference's own p-adaptation (adapt_hp around given vertices) on a straight periodic QUAD
# mesh; the batched context's path (faces at p_f = max(p_L, p_R)) against it.

# name -> (pde, n, base p, highest p, numerical flux, RK steps, [(x, y, target p), ...]); the volumes around each
# vertex are raised to its target, the rest stay at the base order.
MIXED_CASES = {
    "mx_adv_n8": ("advection", 8, 2, 4, 11, 20, [(-0.5, -0.5, 4), (0.5, 0.5, 3), (0.0, -0.75, 3), (-0.75, 0.5, 4)]),
    "mx_euler_n8": ("euler", 8, 1, 3, 31, 10, [(2.5, 2.5, 3), (7.5, 7.5, 2), (5.0, 1.25, 2), (1.25, 7.5, 3)]),
    # the Taylor-Couette case of "tc_n2" (rotating inner wall, adiabatic outer wall, BR2, Roe-Pike) on its parametric
    # square annulus (vertices in the square's coordinates)
    "mx_tc_n2": ("navier_stokes_tc", 2, 2, 4, 31, 10, [(-0.75, 0.0, 4), (0.75, 0.75, 3)]),
    # the Euler supersonic vortex of "sv_n3" (Riemann faces with the exact solution outside, slip walls on both arcs)
    # on its parametric quarter square annulus
    "mx_sv_n3": ("euler_sv", 3, 2, 4, 31, 10, [(0.376, 1.128, 4), (1.256, 1.256, 3)]),
    # the subsonic duct of "duct_n4" (total T/p inflow, back-pressure outflow, slip walls) on its straight box
    "mx_duct_n4": ("euler_duct", 4, 2, 4, 31, 10, [(2.5, 2.5, 4), (7.5, 5.0, 3)]),
    # the same box at Mach 1.5 with supersonic inflow and outflow ("sduct_n4")
    "mx_sduct_n4": ("euler_sduct", 4, 2, 4, 31, 10, [(5.0, 2.5, 4), (2.5, 7.5, 3)]),
    # the steady advection case with its source term (steady/default, "c1_source_bc") on a straight 6^2 box of
    # [-1,1]^2 with upwind faces on its four sides (the steady solution outside)
    "mx_src_n6": ("advection_default_bc", 6, 2, 4, 11, 20, [(0.0, 0.0, 4), (-2.0 / 3.0, 1.0 / 3.0, 3)]),
}


def _mixed_box(pde):
    return (-1.0, 1.0) if pde == "advection" else (0.0, 10.0)


def host_mixed_problem(name: str, p_vol, face_vol=None, face_lf=None):
    """The repo's own mixed-order set-up of a case with the orders p_vol (the reference's, after its adaptation):
    a straight periodic QUAD mesh, the case's state at every volume's solution nodes, dt from the CFL estimate.

    face_vol / face_lf: the reference's face list after adaptation. It keeps the structured mesh's faces in the same
    order, but the faces it rebuilt around adapted volumes may list their two sides the other way round; the mesh
    takes those sides (checked to be the same two volumes and local faces)."""
    from dpgsolver_gb300.host import mixed as M
    from dpgsolver_gb300.host.mesh import StructuredMesh
    from dpgsolver_gb300.host import problem as P
    pde, n, p, p_max, flux, steps, _ = MIXED_CASES[name]
    if pde == "navier_stokes_tc":
        from dpgsolver_gb300.host.gmsh import GmshMesh, GmshTPMesh
        mesh = GmshTPMesh(GmshMesh(_tc_mesh(name, n, False), 2))
    elif pde == "euler_sv":
        from dpgsolver_gb300.host.gmsh import GmshMesh, GmshTPMesh
        mesh = GmshTPMesh(GmshMesh(_case_mesh(name, lambda path: _sv_mesh(path, n)), 2))
    elif pde in ("euler_duct", "euler_sduct"):
        mesh = StructuredMesh(2, n, 0.0, 10.0, periodic=(False, False))
    elif pde == "advection_default_bc":
        mesh = StructuredMesh(2, n, -1.0, 1.0, periodic=(False, False))
    else:
        lo, hi = _mixed_box(pde)
        mesh = StructuredMesh(2, n, lo, hi)
    if face_vol is not None:
        fv, fl = np.asarray(face_vol), np.asarray(face_lf)
        same = np.all(fv == mesh.face_vol, axis=1) & np.all(fl == mesh.face_lf, axis=1)
        swap = np.all(fv == mesh.face_vol[:, ::-1], axis=1) & np.all(fl == mesh.face_lf[:, ::-1], axis=1)
        if fv.shape != mesh.face_vol.shape or not np.all(same | swap):
            raise AssertionError("face lists differ")
        mesh.face_vol = fv.astype(mesh.face_vol.dtype)
        mesh.face_lf = fl.astype(mesh.face_lf.dtype)
    if pde == "navier_stokes_tc":
        prob = M.MixedTPProblem(name, 2, P.PDE_NAVIER_STOKES, flux, True, np.zeros(3), mesh, p_vol,
                                parametric=P.cylinder_parametric_map)
        prob.ns = dict(P._ns_params(_TC_MU, Pr=0.72, r_s=1.0), dTdn=0.0)
        fn = lambda x: _tc_state(x, False)   # noqa: E731
    elif pde == "euler_sv":
        prob = M.MixedTPProblem(name, 2, P.PDE_EULER, flux, True, np.zeros(3), mesh, p_vol,
                                parametric=P.cylinder_parametric_map)
        fn = _sv_state
    elif pde == "advection_default_bc":
        prob = M.MixedTPProblem(name, 2, P.PDE_ADVECTION, flux, False, np.array([1.0, 0.5, 0.0]), mesh, p_vol)
        fn = _advection_default_state
    elif pde in ("euler_duct", "euler_sduct"):
        prob = M.MixedTPProblem(name, 2, P.PDE_EULER, flux, True, np.zeros(3), mesh, p_vol)
        fn = _duct_state if pde == "euler_duct" else _sduct_state
    elif pde == "advection":
        prob = M.MixedTPProblem(name, 2, P.PDE_ADVECTION, flux, False, np.array([1.0, 0.5, 0.0]), mesh, p_vol)
        fn = _advection_state
    else:
        prob = M.MixedTPProblem(name, 2, P.PDE_EULER, flux, True, np.zeros(3), mesh, p_vol)
        fn = _vortex_state
    for g in range(len(prob.groups)):
        if len(prob.group_vols[g]):
            x = prob.solution_node_xyz(g)
            U = np.asarray(fn(x.reshape(-1, 2))).reshape(x.shape[0], x.shape[1], -1)
            prob.set_group(prob.sol, g, np.transpose(U, (0, 2, 1)))
    prob.dt = prob.stable_dt()
    if pde == "navier_stokes_tc":
        prob.set_boundaries(None, P._taylor_couette_wall(0.5, 1.0, 1.0))
    elif pde == "euler_sv":   # the Riemann faces' exterior state: the exact solution
        prob.set_boundaries(None, lambda xy: np.asarray(P.supersonic_vortex_state(xy[:, 0], xy[:, 1], 1.0)).T)
    elif pde == "euler_duct":   # as P.euler_subsonic_duct: the unperturbed Mach 0.4 stream's BC data
        T_tot = 1.0 + 0.5 * P.GM1 * 0.4 ** 2
        prob.bc_data = (1.0, T_tot, T_tot ** (P.GAMMA / P.GM1), 1.0)
        prob.set_boundaries({(0, 0): P.BC_TOTAL_TP, (0, 1): P.BC_BACKPRESSURE, (1, 0): P.BC_SLIPWALL,
                             (1, 1): P.BC_SLIPWALL},
                            P._uniform_flow(2, 1.0, (0.4 * np.sqrt(P.GAMMA), 0.0), 1.0))
    elif pde == "advection_default_bc":   # as P.advection_default_2d: s = b . grad u at the cubature nodes
        blocks = [None] * prob.n_volumes
        for g, vols in enumerate(prob.group_vols):
            if len(vols) == 0:
                continue
            x, y = prob.geoms[g].xyz_vc[..., 0], prob.geoms[g].xyz_vc[..., 1]
            m, a = P.SOURCE_M, P.SOURCE_A
            src = 1.0 * m * np.cos(m * x + a) * np.sin(m * y + a) + 0.5 * m * np.sin(m * x + a) * np.cos(m * y + a)
            for k, v in enumerate(vols):
                blocks[v] = src[k]
        prob.source_vc = np.concatenate(blocks)
        prob.set_boundaries({(dd, sd): P.BC_UPWIND for dd in range(2) for sd in range(2)},
                            lambda xy: np.asarray(_advection_default_state(xy)).reshape(len(xy), 1))
    elif pde == "euler_sduct":   # as P.euler_supersonic_duct_2d: the unperturbed Mach 1.5 stream outside
        prob.bc_data = (0.0, 0.0, 0.0, 0.0)
        prob.set_boundaries({(0, 0): P.BC_SUPERSONIC_IN, (0, 1): P.BC_SUPERSONIC_OUT, (1, 0): P.BC_SLIPWALL,
                             (1, 1): P.BC_SLIPWALL},
                            P._uniform_flow(2, 1.0, (1.5 * np.sqrt(P.GAMMA), 0.0), 1.0))
    return prob


def run_mixed(name: str) -> dict:
    """Run a mixed-order case through the reference: its adaptation decides every volume's order; the host problem
    with those orders gives the state formula's values and dt. Returns the flat arrays of the fixture."""
    pde, n, p, p_max, flux, steps, adapt = MIXED_CASES[name]
    if pde == "navier_stokes_tc":
        from dpgsolver_gb300.host.gmsh import write_square_annulus_msh
        ns = dict(_tc_ns(), dTdn=0.0, omega=1.0, p_b=1.0, t_b=1.0, rho_b=1.0, E_b=1.0 / 0.4 + 0.5 * 0.5 ** 2)
        extra = dict(mesh_writer=lambda path: write_square_annulus_msh(path, n, n, outer=20111), ns=ns)
        run = lambda **kw: run_case(name, "navier_stokes", n, p, 0.0, 1.0, flux, adapt_p=adapt,   # noqa: E731
                                    p_max=p_max, **extra, **kw)
        out0 = run()
        p_vol = out0["volumes"][:, 2].astype(np.int32)
        prob = host_mixed_problem(name, p_vol, out0["faces"][:, [4, 7]], out0["faces"][:, [5, 8]])
        out = run(states_fn=lambda o: [_tc_state(x, False) for x in o["xyz_vs"]], steps=steps, dt=prob.dt)
        return _mixed_arrays(name, p_vol, n, flux, steps, prob, out)
    if pde == "advection_default_bc":
        from dpgsolver_gb300.host.gmsh import write_box_msh
        codes = {(k, s_): 10041 for k in range(2) for s_ in range(2)}
        extra = dict(mesh_writer=lambda path: write_box_msh(path, 2, n, lo=-1.0, hi=1.0, periodic=False, codes=codes),
                     pde_spec="steady/default")
        run = lambda **kw: run_case(name, "advection", n, p, -1.0, 1.0, flux, adapt_p=adapt,   # noqa: E731
                                    p_max=p_max, **extra, **kw)
        out0 = run()
        p_vol = out0["volumes"][:, 2].astype(np.int32)
        prob = host_mixed_problem(name, p_vol, out0["faces"][:, [4, 7]], out0["faces"][:, [5, 8]])
        out = run(state_fn=_advection_default_state, steps=steps, dt=prob.dt)
        return _mixed_arrays(name, p_vol, n, flux, steps, prob, out)
    if pde in ("euler_duct", "euler_sduct"):
        from dpgsolver_gb300.host.gmsh import write_box_msh
        sup = pde == "euler_sduct"
        codes = {(0, 0): 10105 if sup else 10104, (0, 1): 10106 if sup else 10103, (1, 0): 10102, (1, 1): 10102}
        prob0 = host_mixed_problem(name, np.full(n * n, p, dtype=np.int32))
        extra = dict(mesh_writer=lambda path: write_box_msh(path, 2, n, lo=0.0, hi=10.0, periodic=False, codes=codes),
                     pde_spec="steady/free_stream", bc_data=prob0.bc_data, mach=1.5 if sup else 0.4)
        run = lambda **kw: run_case(name, "euler", n, p, 0.0, 10.0, flux, adapt_p=adapt,   # noqa: E731
                                    p_max=p_max, **extra, **kw)
        out0 = run()
        p_vol = out0["volumes"][:, 2].astype(np.int32)
        prob = host_mixed_problem(name, p_vol, out0["faces"][:, [4, 7]], out0["faces"][:, [5, 8]])
        out = run(state_fn=_sduct_state if sup else _duct_state, steps=steps, dt=prob.dt)
        return _mixed_arrays(name, p_vol, n, flux, steps, prob, out)
    if pde == "euler_sv":
        extra = dict(mesh_writer=lambda path: _sv_mesh(path, n), pde_spec="steady/supersonic_vortex")
        run = lambda **kw: run_case(name, "euler", n, p, 0.0, 1.0, flux, adapt_p=adapt,   # noqa: E731
                                    p_max=p_max, **extra, **kw)
        out0 = run()
        p_vol = out0["volumes"][:, 2].astype(np.int32)
        prob = host_mixed_problem(name, p_vol, out0["faces"][:, [4, 7]], out0["faces"][:, [5, 8]])
        out = run(states_fn=lambda o: [_sv_state(x) for x in o["xyz_vs"]], steps=steps, dt=prob.dt)
        return _mixed_arrays(name, p_vol, n, flux, steps, prob, out)
    lo, hi = _mixed_box(pde)
    fn = _advection_state if pde == "advection" else _vortex_state
    out0 = run_case(name, pde, n, p, lo, hi, flux, adapt_p=adapt, p_max=p_max)
    p_vol = out0["volumes"][:, 2].astype(np.int32)
    prob = host_mixed_problem(name, p_vol, out0["faces"][:, [4, 7]], out0["faces"][:, [5, 8]])
    out = run_case(name, pde, n, p, lo, hi, flux, state_fn=lambda x: np.asarray(fn(x)).reshape(len(x), -1),
                   steps=steps, dt=prob.dt, adapt_p=adapt, p_max=p_max)
    return _mixed_arrays(name, p_vol, n, flux, steps, prob, out)


def _tc_ns() -> dict:
    """The Navier-Stokes constants of the Taylor-Couette cases (mu, Pr = 0.72, r_s = 1, constant viscosity)."""
    from dpgsolver_gb300.host import problem as P
    return P._ns_params(_TC_MU, Pr=0.72, r_s=1.0)


def _mixed_arrays(name, p_vol, n, flux, steps, prob, out) -> dict:
    """The flat arrays of a mixed-order fixture from the reference's run."""
    case_dir = os.path.join(RUN_DIR, name)
    raw = lambda f: _read_bin(os.path.join(case_dir, f))   # noqa: E731
    mx = np.loadtxt(os.path.join(case_dir, "max_rhs.txt"), ndmin=1)
    return dict(p_vol=p_vol, n=np.int64(n), num_flux=np.int64(flux), steps=np.int64(steps), dt=np.float64(prob.dt),
                face_vol=out["faces"][:, [4, 7]].astype(np.int32), face_lf=out["faces"][:, [5, 8]].astype(np.int32),
                face_ord=out["faces"][:, [6, 9]].astype(np.int32), n_fc=out["faces"][:, 3].astype(np.int32),
                xyz_vs=np.concatenate([x.ravel() for x in out["xyz_vs"]]),
                metrics_vc=raw("metrics_vc.bin"), jacobian_det_vc=raw("jacobian_det_vc.bin"),
                normals_fc=raw("normals_fc.bin"), jacobian_det_fc=raw("jacobian_det_fc.bin"),
                sol_in=out["sol_in"], rhs=out["rhs"], max_rhs=np.float64(mx[0]),
                sol_steps=out["sol_steps"], max_rhs_steps=mx[1:])


# After its adaptation the reference's geometry of some volumes of the supersonic vortex case differs from the map
# evaluated afresh at their new order (3 of its 18 volumes, by up to 1.2e-4); the volume lists are matched by their
# nodes to that tolerance there, and the reference's own geometry is used.
_XYZ_TOL = {"mx_sv_n3": 1e-3}
# Cases whose residual is held to 4 x its one-ulp floor instead of 2 x: the energy residual of p = 4 volumes next to
# lower orders and walls, where the operators of the factored forms (and the oracle's own) round differently from the
# reference's (measured: oracle 2.5 x and GPU 2.3 x the floor).
WIDE_FLOOR = {"mx_sv_n3", "mx_tc_n2"}


def with_reference_mixed_inputs(prob, ref: dict):
    """The mixed-order host problem given the reference's geometry and initial state (flat layouts), after checking
    that both list the same volumes (orders and solution nodes) and faces in the same order."""
    if not np.array_equal(prob.p_vol, ref["p_vol"]):
        raise AssertionError("orders differ")
    xyz = np.concatenate([prob.solution_node_xyz(g)[k].ravel()
                          for v in range(prob.n_volumes)
                          for g in [prob.vol_group[v]]
                          for k in [int(np.nonzero(prob.group_vols[g] == v)[0][0])]])
    if np.abs(xyz - ref["xyz_vs"]).max() > _XYZ_TOL.get(prob.name, 1e-12):
        raise AssertionError("volume lists differ")
    interior = ref["face_vol"][:, 1] >= 0
    if not (np.array_equal(prob.mesh.face_vol, ref["face_vol"]) and np.array_equal(prob.mesh.face_lf, ref["face_lf"])
            and not np.any(ref["face_ord"][interior]) and np.array_equal(np.diff(prob.face_off), ref["n_fc"])):
        raise AssertionError("face lists differ")
    flat = prob.flat
    prob.sol = np.array(ref["sol_in"], dtype=np.float64)

    def ref_flat():
        fl = flat()
        fl.update(metrics_vc=np.array(ref["metrics_vc"]), jacobian_det_vc=np.array(ref["jacobian_det_vc"]),
                  normals_fc=np.array(ref["normals_fc"]), jacobian_det_fc=np.array(ref["jacobian_det_fc"]),
                  sol=prob.sol)
        return fl
    prob.flat = ref_flat
    return prob
