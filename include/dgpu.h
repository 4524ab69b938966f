/* dgpu.h -- C ABI of the GB300 (sm_103a) explicit DG residual for DPGSolver.
 *
 * Plain C, no C++ or CUDA types in any signature. Every entry returns a dgpu_status (DGPU_OK == 0); the
 * library never aborts. All device memory is owned by the opaque context; one CUDA stream per context; no
 * global state, so separate contexts may be used from separate host threads.
 *
 * Entry points and the reference interface each one replaces (paths inside DPGSolver):
 *   dgpu_create            set-up of the DG solver volumes/faces that solve_explicit performs before its time loop:
 *                          constructor_derived_computational_elements(IL_SOLVER_DG) and the inverse mass matrices
 *                          (src/simulation/solvers/solve_explicit.c:86-89,
 *                           src/simulation/solvers/dg/volume_solver_dg_T.c:49-78)
 *   dgpu_upload_state      writes every Solver_Volume_T::sol_coef (src/simulation/solvers/volume_solver_T.h:31-104)
 *   dgpu_download_state    reads them back
 *   dgpu_compute_rhs       double compute_rhs_dg(const struct Simulation*)  (src/simulation/solvers/dg/solve_dg.c:130-136)
 *                          = compute_volume_rlhs_dg (compute_volume_rlhs_dg.h) + compute_face_rlhs_dg
 *                          (compute_face_rlhs_dg.h) + scale_rhs_by_m_inv + compute_max_rhs_dg_like
 *   dgpu_download_rhs      reads every Solver_Volume_T::rhs
 *   dgpu_compute_rhs_host  compute_rhs_dg with host sol_coef in and host rhs out (one call, copies included)
 *   dgpu_ssp_rk3_step      static double time_step_ssp_rk_33(double dt, const struct Simulation*)
 *                          (src/simulation/solvers/solve_explicit.c:252-301), positivity included
 *                          (enforce_positivity_highorder, src/simulation/solvers/solve.c:187-233)
 *   dgpu_ssp_rk3_steps     n_steps iterations of the time loop body of solve_explicit (solve_explicit.c:92-112)
 */
#ifndef DGPU_H
#define DGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int dgpu_status;
#define DGPU_OK                   0
#define DGPU_ERR_INVALID_ARGUMENT 1  /* a NULL, size or index out of range                                  */
#define DGPU_ERR_UNSUPPORTED      2  /* element type, order, PDE or flux not provided by this library        */
#define DGPU_ERR_CUDA             3  /* a CUDA runtime call failed (dgpu_last_error names it)                */
#define DGPU_ERR_POSITIVITY       4  /* average density or pressure below EPS_PHYS (reference: EXIT_ERROR,
                                        src/simulation/solvers/solve.c:204-208)                             */
#define DGPU_ERR_NO_DEVICE        5  /* no CUDA device of compute capability 10.3                            */

/* PDE, numerical flux and element codes: the reference's own values
 * (src/simulation/test_case/definitions_test_case.h, src/simulation/solvers/numerical_flux/
 *  definitions_numerical_flux.h, src/element/definitions_elements.h). */
#define DGPU_PDE_ADVECTION 1
#define DGPU_PDE_EULER     3
#define DGPU_PDE_NAVIER_STOKES 4   /* Euler flux + viscous flux, BR2 second-order terms (QUAD/HEX volumes) */
#define DGPU_VISCOSITY_CONSTANT   101   /* definitions_physics.h:34-36 */
#define DGPU_VISCOSITY_SUTHERLAND 102
#define DGPU_NUM_FLUX_UPWIND          11
#define DGPU_NUM_FLUX_ROE_PIKE        31
#define DGPU_NUM_FLUX_LAX_FRIEDRICHS  32
#define DGPU_TRI   2
#define DGPU_QUAD  3
#define DGPU_TET   4
#define DGPU_HEX   5
#define DGPU_WEDGE 6
#define DGPU_PYR   7

typedef struct dgpu_ctx dgpu_ctx;

/* Test-case parameters (Test_Case_T fields pde_index, num_flux_1st, and the advection velocity of
 * solution_advection_T.c; constant velocity only). */
typedef struct {
	int d;              /* 2 or 3 (the reference's compile-time DIM)                       */
	int pde;            /* DGPU_PDE_*                                                       */
	int num_flux;       /* DGPU_NUM_FLUX_*                                                  */
	int positivity;     /* 1: enforce_positivity_highorder after every RK stage (Euler)     */
	double b_adv[3];    /* advection velocity (advection only)                              */
	/* Navier-Stokes only, the test case's constants the reference reads from its input file
	 * (solution_navier_stokes_T.c:188-255, flux_navier_stokes_T.c:461-482): the viscosity model
	 * (DGPU_VISCOSITY_CONSTANT: mu; DGPU_VISCOSITY_SUTHERLAND: 0.08 mu sqrt(T) / (1 + 112 / T), T = p / (rho r_s)),
	 * mu, the Prandtl number and the specific gas constant. The inviscid numerical flux is num_flux; the second-order
	 * one is BR2 (NUM_FLUX_BR2_STABLE: central flux of the partially corrected gradients, scaling 1.01 * 2d), the only
	 * explicit DG option of the reference. */
	int viscosity;
	double mu, Pr, r_s;
	/* BC_NOSLIP_DIABATIC walls: the normal temperature gradient dTdn of the input (diabatic_flux_type constant;
	 * 0 for constant_zero). The wall's normal energy flux is -mu Cp / Pr dTdn, Cp = gamma / (gamma - 1) r_s
	 * (get_normal_flux_Energy, solution_navier_stokes.c:93-150); a non-zero dTdn needs constant viscosity. */
	double dTdn;
} dgpu_physics;

/* Tensor-product operator set of one (element type, p): the 1D factors of the reference's Operator::ops_tp
 * (src/simulation/operators/operator.h:40-44) for the solution basis (Lagrange on GLL nodes, q = p+1) and
 * the GL cubature (q points). All matrices row-major. */
typedef struct {
	int elem_type;               /* DGPU_QUAD or DGPU_HEX                                      */
	int p;                       /* 1..4                                                       */
	const double* cv0_vs_vc;     /* (q x q): basis at the volume cubature nodes                */
	const double* cv1_vs_vc;     /* (q x q): first derivative at the volume cubature nodes     */
	const double* cv0_vs_fc;     /* (2 x q): basis at r = -1 and r = +1                        */
	const double* w_vc;          /* (q):     GL cubature weights                               */
	const double* ccSB0_vs_vs;   /* (q x q): Lagrange -> Bezier coefficients (positivity)      */
	const double* ccBS0_vs_vs;   /* (q x q): Bezier -> Lagrange coefficients (positivity)      */
} dgpu_tp_operators;

/* Geometry and connectivity packed from the Solver_Volume / Solver_Face lists in list order. */
typedef struct {
	int n_volumes;
	const double* metrics_vc;      /* n_volumes x (n_vc, d, d) column-major: Solver_Volume_T::metrics_vc */
	const double* jacobian_det_vc; /* n_volumes x n_vc: Solver_Volume_T::jacobian_det_vc                */
	int n_faces;
	const int* face_vol;           /* n_faces x 2: volume index of neigh_info[0] / neigh_info[1]        */
	const int* face_lf;            /* n_faces x 2: neigh_info[s].ind_lf                                 */
	const int* nc_fc;              /* n_faces x n_fc or NULL: right-trace gather permutation
	                                  (get_operator__nc_fc_T(1, face), compute_face_rlhs_T.c:133-146);
	                                  NULL means the identity for every face                           */
	const double* normals_fc;      /* n_faces x (n_fc x d) row-major: Solver_Face_T::normals_fc         */
	const double* jacobian_det_fc; /* n_faces x n_fc: Solver_Face_T::jacobian_det_fc                    */
	/* Boundary faces: face_vol[2f+1] = -1 (no neighbour; the face belongs to its side-0 volume, normals_fc
	 * outward from it). Both arrays may be NULL when no face is a boundary face.
	 * bc_fc: n_faces: Face::bc, the reference's BC code (definitions_bc.h), read on boundary faces only and
	 *   taken modulo BC_STEP_SC = 10000. Euler: BC_RIEMANN 101, BC_SLIPWALL 102, BC_BACKPRESSURE 103,
	 *   BC_TOTAL_TP 104, BC_SUPERSONIC_IN 105, BC_SUPERSONIC_OUT 106 (boundary_euler_T.c); advection:
	 *   inflow/outflow/upwind 1-3, 11-13, 41-46, all the upwind boundary value (boundary_advection_T.c:40-77);
	 *   Navier-Stokes: BC_RIEMANN, BC_SUPERSONIC_IN, BC_SUPERSONIC_OUT (with the interior gradient),
	 *   BC_NOSLIP_ADIABATIC 111 and BC_NOSLIP_DIABATIC 112 (static walls, boundary_navier_stokes_T.c:130-156,
	 *   258-304) and BC_NOSLIP_ALL_ROTATING 113 (boundary_navier_stokes_T.c:117-128, 196-244).
	 *   Other codes: DGPU_ERR_UNSUPPORTED.
	 * bc_state_fc: n_faces x (n_fc x n_var) row-major: the test case's conserved solution at the face's
	 *   cubature nodes (constructor_sol_bv(xyz_fc)), the exterior data of Riemann, supersonic inflow and
	 *   upwind inflow boundaries; on BC_NOSLIP_ALL_ROTATING faces the wall state (rho_b, rho_b u_wall, E_b) with
	 *   the wall's velocity at the node (compute_uvw_ex_rotating: omega about the z axis); read on boundary
	 *   faces only.
	 * dgpu_create and the batched context (Euler and advection codes; there the boundary face's nodes are those of
	 *   its side-0 volume's order); the no-allocation entry returns DGPU_ERR_UNSUPPORTED. */
	const int* bc_fc;
	const double* bc_state_fc;
	/* bc_data: 4 doubles {p_back, t_total, p_total, r_s}, the reference's BC_Data (boundary_euler_T.c:44-49, read
	 * from the test case's input file there) for BC_BACKPRESSURE and BC_TOTAL_TP faces; NULL when none. */
	const double* bc_data;
	/* Geometry coefficients instead of the four geometric factor arrays (metrics_vc, jacobian_det_vc, normals_fc,
	 * jacobian_det_fc all NULL): the device computes the factors (set_up_solver_geometry_T, geometry_T.c:165-185).
	 * geom_coef: n_volumes x (n_g x d) column-major, Solver_Volume_T::geom_coef: the coordinates at the GLL nodes
	 * of order p_g (n_g = (p_g+1)^d, first direction fastest); p_g = p for curved volumes, 1 for straight ones
	 * (geometry_T.c:740-742). NULL when the factors are given. dgpu_create only. */
	int p_g;
	const double* geom_coef;
} dgpu_mesh;

/* Create a context on the current CUDA device and copy everything it needs; the caller may free its arrays
 * when this returns. State size = n_volumes * n_var * q^d doubles, per volume the reference's (n_vs x n_var)
 * column-major sol_coef block. */
dgpu_status dgpu_create(const dgpu_physics* phys, const dgpu_tp_operators* ops, const dgpu_mesh* mesh,
                        dgpu_ctx** out);
dgpu_status dgpu_destroy(dgpu_ctx* ctx);

/* Geometry precompute on the device, results in host buffers in dgpu_mesh's layouts (any output may be NULL):
 * set_up_solver_geometry_T (geometry_T.c:165-185) for QUAD (d = 2) / HEX (d = 3) volumes of order ops->p from
 * mesh->geom_coef and mesh->p_g, with the faces' side 0 (mesh->face_vol, face_lf) and their cubature nodes:
 *   metrics_vc      n_volumes x (n_vc, d, d) column-major: the vm metric terms (2D cofactors, compute_cofactors_T
 *                   geometry_T.c:546-590; 3D the conservative curl form) interpolated to the GL nodes (:734-801);
 *   jacobian_det_vc n_volumes x n_vc: det of the Jacobian evaluated at the GL nodes;
 *   normals_fc      n_faces x (n_fc x d) row-major, jacobian_det_fc n_faces x n_fc: side 0's vm metric terms at
 *                   the face nodes times the reference normal, normalised / its length (:274-325, :412-445);
 *   xyz_fc          n_faces x (n_fc x d) row-major: the face cubature nodes' coordinates (for constructor_sol_bv).
 * Synchronous. DGPU_ERR_INVALID_ARGUMENT when a Jacobian determinant is not positive. Of ops only elem_type, p and
 * w_vc are read. */
/* Blended geometry coefficients of curved QUAD volumes on the device, host buffers in and out (synchronous): the
 * reference's compute_geom_coef_blended_T (geometry_T.c:845-855, constructor_xyz_blended_ce
 * geometry_blended_T.c:286-315) with TP Gordon-Hall blending and the radial projection of its blended n-cylinder
 * domains (constructor_xyz_surface_cylinder_radial_proj_T, geometry_surface_T.c:103-147: each curved face's straight
 * nodes moved to the circle about the origin through the face's first vertex).
 *   xyz_ve      n_volumes x (4 x 2) column-major: the straight volume's vertices (Volume::xyz_ve, TP order; the
 *               p_g = 1 geom_coef layout);
 *   face_curved n_volumes x 4: 1 where local face lf (element.c order) is a curved boundary face
 *               (Face::bc > BC_CURVED_START = 20000, is_face_bc_curved), else 0;
 *   geom_coef   out, n_volumes x ((p_g+1)^2 x 2) column-major: the coordinates at the GLL nodes of order p_g, the
 *               layout of dgpu_mesh.geom_coef.
 * d = 2 only: the reference's 3D TP blending stops with EXIT_ADD_SUPPORT, and its other parametrizations
 * (arc_length, normal_proj) are EXIT_ADD_SUPPORT too. Volumes without a curved face get the bilinear map. */
dgpu_status dgpu_blend_geometry(int d, int p_g, int n_volumes, const double* xyz_ve, const int* face_curved,
                                double* geom_coef);
dgpu_status dgpu_compute_geometry(int d, const dgpu_tp_operators* ops, const dgpu_mesh* mesh, double* metrics_vc,
                                  double* jacobian_det_vc, double* normals_fc, double* jacobian_det_fc,
                                  double* xyz_fc);

dgpu_status dgpu_state_size(const dgpu_ctx* ctx, size_t* n_doubles);
dgpu_status dgpu_upload_state(dgpu_ctx* ctx, const double* sol);      /* host -> device, synchronous */
dgpu_status dgpu_download_state(dgpu_ctx* ctx, double* sol);          /* device -> host, synchronous */
dgpu_status dgpu_download_rhs(dgpu_ctx* ctx, double* rhs);            /* device -> host, synchronous */

/* Residual of the device state into the device rhs (M^-1 applied). max_rhs may be NULL (then nothing is
 * synchronised); otherwise it receives max |rhs| after the stream finishes. */
dgpu_status dgpu_compute_rhs(dgpu_ctx* ctx, double* max_rhs);
/* Same with host buffers: sol (host) -> device, residual, device -> rhs (host). */
dgpu_status dgpu_compute_rhs_host(dgpu_ctx* ctx, const double* sol, double* rhs, double* max_rhs);

/* One SSP-RK3 step on the device state (three residuals, stage updates and positivity), replayed from a CUDA
 * graph captured on first use for each dt. max_rhs: as for dgpu_compute_rhs (last stage's residual). */
dgpu_status dgpu_ssp_rk3_step(dgpu_ctx* ctx, double dt, double* max_rhs);
dgpu_status dgpu_ssp_rk3_steps(dgpu_ctx* ctx, double dt, int n_steps, double* max_rhs);
/* time_step_ssp_rk_33 (solve_explicit.c:252-301) on host state: sol_in (host, the sol_coef blocks) -> one SSP-RK3
 * step -> sol_out (host; may equal sol_in), synchronous; the device state becomes the new state. The same result,
 * bit for bit, as dgpu_upload_state + dgpu_ssp_rk3_step + dgpu_download_state. For page-locked buffers
 * (cudaHostAlloc / cudaHostRegister) the transfers happen inside the step's first volume kernel and last lift
 * kernel, overlapped with their arithmetic; pageable buffers are copied. Replayed from a CUDA graph captured for
 * each (dt, buffers, max_rhs requested); Navier-Stokes contexts run the three calls above. */
dgpu_status dgpu_ssp_rk3_step_host(dgpu_ctx* ctx, double dt, const double* sol_in, double* sol_out,
                                   double* max_rhs);

/* Residual without any device allocation. No counterpart in the reference (its residual is host code).
 *
 * For callers that cannot call cudaMalloc: a host application whose GPU memory belongs to its own pool or
 * framework and which passes the library only the buffers it owns, or a loop that must not allocate while it
 * runs. It computes what dgpu_compute_rhs computes, from a context-free description: `phys` and `ops` are host
 * structs as for dgpu_create, while every array in `d_mesh` (same layouts as dgpu_create), `d_sol` and
 * `d_rhs` must be device memory of the current device. The intermediates live in one fixed array of
 * DGPU_NOALLOC_SCRATCH_BYTES inside the library (held by every GPU that loads it until the process exits);
 * a mesh that needs more returns DGPU_ERR_INVALID_ARGUMENT naming the size it needs (a HEX p=3 Euler element
 * needs about 15 KB, so about 2,200 such elements fit). The first call on each device looks up the array's
 * device address, so make that first call before any stream capture. All calls share the array and each
 * call overwrites it: calls that overlap on the GPU (concurrent streams or host threads) race, so serialise
 * them. The call synchronises `cuda_stream` (NULL = legacy default stream) after validating the mesh on the
 * device, and again when max_rhs is not NULL. */
#define DGPU_NOALLOC_SCRATCH_BYTES (32u << 20)
dgpu_status dgpu_compute_rhs_noalloc(const dgpu_physics* phys, const dgpu_tp_operators* ops,
                                     const dgpu_mesh* d_mesh, const double* d_sol, double* d_rhs,
                                     double* max_rhs, void* cuda_stream);

/* Discrete adjoint of the residual, as a forward/backward pair shaped like an autograd Function.
 * dgpu_vjp_forward computes R(sol) exactly as dgpu_compute_rhs_host does and keeps sol on the device;
 * dgpu_vjp_backward returns grad = (dR/dsol)^T cotangent at that state (host buffers, state layout). The reference
 * has no adjoint: it linearises the same residual by complex step (compute_lhs_cmplx_step_dg,
 * src/testing/support/simulation/solvers/dg/test_support_solve_dg.c:83-110) and assembles its Jacobian for the
 * implicit solver (compute_rlhs_dg, src/simulation/solvers/dg/solve_dg.c:138-145); grad is that Jacobian's
 * transpose applied to the cotangent. Kinks of the fluxes take the derivative of the branch the value takes.
 * Every PDE: for Navier-Stokes the BR2 gradients, their liftings, the viscous fluxes and the boundary values (walls
 * included) are differentiated with the rest. */
dgpu_status dgpu_vjp_forward(dgpu_ctx* ctx, const double* sol, double* rhs, double* max_rhs);
dgpu_status dgpu_vjp_backward(dgpu_ctx* ctx, const double* cotangent, double* grad_sol);

/* Forward-mode linearisation (the matrix-free Jacobian-vector product of an implicit solver): rhs = R(sol) (may be
 * NULL) and jv = (dR/dsol) dir, host buffers in the state layout; the context's state becomes sol. The reference
 * forms the same product by complex step (compute_lhs_cmplx_step_dg, src/testing/support/simulation/solvers/dg/
 * test_support_solve_dg.c:83-110) and assembles the Jacobian itself for its implicit solver (compute_rlhs_dg,
 * src/simulation/solvers/dg/solve_dg.c:138-145); here the flux routines run on dual numbers, which gives the
 * product without a step size. Kinks of the fluxes take the derivative of the branch the value takes. Every PDE,
 * Navier-Stokes included (its gradients, liftings and viscous flux are linearised with the rest). */
dgpu_status dgpu_jvp(dgpu_ctx* ctx, const double* sol, const double* dir, double* rhs, double* jv);

/* Block-sparse Jacobian of the residual at sol, the matrix the reference assembles for its implicit solver block by
 * block (constructor_lhs_v_1_T, compute_volume_rlhs_T.c:179-220; constructor_lhs_f_1_T, compute_face_rlhs_T.c:163-220)
 * and adds to PETSc (add_to_petsc_Mat, solve.c:321-338). Block row v = volume v; its blocks are the volume itself
 * and its face neighbours, ascending, each once (boundary faces couple nothing). A block is block_size x block_size,
 * block_size = n_var * n_vs, row-major, row eq * n_vs + i (residual of equation eq at basis function i), column
 * var * n_vs + j: the reference's lhs layout. raw = 1: the derivative of the residual before M^-1 (the reference's
 * lhs, whose right-hand side compute_rlhs_dg leaves unscaled); raw = 0: of the explicit right-hand side
 * (M^-1 applied, the operator of dgpu_compute_rhs and dgpu_jvp).
 * dgpu_jacobian_structure: block_size, the number of blocks and of colours (any output may be NULL); the structure
 *   and the colouring are built on the first call of either entry and kept.
 * dgpu_jacobian_bsr: sol (host, state layout) becomes the context's state; row_ptr (n_volumes + 1), col_idx
 *   (n_blocks) are host buffers and may be NULL; values (n_blocks * block_size^2 doubles) may be NULL (structure only),
 *   device memory of the context's device (written in place) or host memory (staged through a device buffer of the
 *   same size for the call). Computed as n_colours * block_size directional derivatives of the JVP kernels, one per
 *   (colour, local unknown), each giving one column of every block whose column volume has that colour. */
dgpu_status dgpu_jacobian_structure(dgpu_ctx* ctx, int* block_size, long long* n_blocks, int* n_colours);
dgpu_status dgpu_jacobian_bsr(dgpu_ctx* ctx, const double* sol, int raw, int* row_ptr, int* col_idx,
                              double* values);

/* Output functional for the adjoint: J(sol) = sum over the listed faces of the integral of pressure on side 0
 * (sum over face cubature nodes of w_fc J_fc p(W_L)), e.g. the faces of the plane z = 0. Euler and Navier-Stokes. The
 * reference computes such integrals as error functionals (src/simulation/test_case/compute_error/) but has no
 * adjoint; no counterpart. */
dgpu_status dgpu_set_objective_faces(dgpu_ctx* ctx, int n_faces, const int* faces);
/* J(sol) and, when dJ_dsol is not NULL, its gradient (host buffers, state layout). */
dgpu_status dgpu_objective(dgpu_ctx* ctx, const double* sol, double* J, double* dJ_dsol);
/* Adjoint of n_steps SSP-RK3 steps of size dt (the stage expressions of time_step_ssp_rk_33,
 * src/simulation/solvers/solve_explicit.c:277-295, without the positivity limiter, whose corrections are not
 * differentiable): J = J(sol_N) with sol_N the state after n_steps steps from sol0, and dJ/dsol0. States are
 * kept every K steps and the K states of a segment and the stage states of each step are recomputed during the
 * backward sweep; K is chosen so that the (checkpoints + segment + 7 work) states fit in budget_bytes of device
 * memory (DGPU_ERR_INVALID_ARGUMENT names the minimum when they cannot). segment_steps receives K (may be
 * NULL). No counterpart in the reference. */
dgpu_status dgpu_adjoint_ssp_rk3(dgpu_ctx* ctx, double dt, int n_steps, size_t budget_bytes, const double* sol0,
                                 double* J, double* dJ_dsol0, int* segment_steps);

/* Number of positivity corrections applied since creation (enforce_positivity_highorder's correct_coef). */
dgpu_status dgpu_positivity_corrections(dgpu_ctx* ctx, long long* n);
/* Kernels this context has launched (graph replays count each kernel node). */
dgpu_status dgpu_kernel_launches(const dgpu_ctx* ctx, long long* n);
/* Synchronise the context's stream. */
dgpu_status dgpu_synchronize(dgpu_ctx* ctx);
/* Run the context's work on the caller's cudaStream_t (passed as void*) instead of its own stream. The
 * caller keeps ownership of the stream; any captured step graph is discarded. No reference counterpart
 * (the reference is serial host code). */
dgpu_status dgpu_set_stream(dgpu_ctx* ctx, void* cuda_stream);
/* Per-kernel timing with CUDA events around every eager launch (steps then run without a graph).
 * dgpu_kernel_time sums the recorded durations of the kernels named `name` ("tp_volume_kernel",
 * "tp_face_kernel", "tp_lift_kernel"). Measurement aids; no reference counterpart. */
dgpu_status dgpu_set_kernel_timing(dgpu_ctx* ctx, int enable);
dgpu_status dgpu_kernel_time(dgpu_ctx* ctx, const char* name, double* total_ms, long long* count);
/* Source term of the test case: compute_source_rhs_dg_like (src/simulation/solvers/compute_rlhs.c:47-57), called by
 * compute_rlhs_common_dg (src/simulation/solvers/dg/solve_dg.c:188), which adds tw0_vt_vc (J_vc s) to every volume's
 * rhs before M^-1 (e.g. compute_source_rhs_advection_default_T, solution_advection_default_T.c:79-94). source_vc:
 * host, per volume (n_vc x n_var) column-major, the test case's source at the volume cubature nodes (what its
 * constructor_source_* returns, before the J scaling), in the state's layout (n_vc = n_vs for these elements); NULL
 * removes it. The values are copied. Every later residual and RK stage of this context includes the source, and so
 * does the primal of the linearisations (their derivatives do not depend on it). */
dgpu_status dgpu_set_source(dgpu_ctx* ctx, const double* source_vc);

/* Text of the last error recorded on this context (or of the last failed dgpu_create when ctx is NULL). */
const char* dgpu_last_error(const dgpu_ctx* ctx);

/* Element partitions across GPUs, one process per GPU: the distributed form of compute_rhs_dg and
 * time_step_ssp_rk_33 (the reference itself runs on one process: src/simulation/simulation.c:360-369 records rank and
 * size only). Each rank creates its context with dgpu_create on its own volumes and every face that has one of
 * them, in the global face order, keeping the global side numbering; a side whose volume belongs to another rank
 * has face_vol = DGPU_REMOTE_VOLUME (its face_lf is ignored). Such a face is an interior face: its remote side's
 * trace arrives by exchange. Both ranks evaluate the face's numerical flux from the same two traces, and each lifts
 * it into its own volume only, so the partitioned residual equals the single-domain one bit for bit.
 * dgpu_halo_setup: the n_slots cut faces (n_slots must equal the number of remote sides), slot = 2 f + side in the
 *   local face list: send_slots[i] the local side of cut face i, recv_slots[i] its remote side. Order them per
 *   neighbour rank in global face order, so that rank A's send list towards B is B's receive list from A.
 * dgpu_halo_buffers: device buffers owned by the context, n_slots x slot_doubles (n_var x n_fc) each: the traces
 *   to send (written by *_begin) and the traces received (read by *_end).
 * One SSP-RK3 step = for stage 0, 1, 2: dgpu_halo_stage_begin (volume term, traces packed into d_send; enqueued on
 * the context's stream, dgpu_get_stream) -> the caller moves every neighbour's d_send block into this rank's
 * d_recv (NCCL send/recv or peer copies, enqueued on that stream or completed before the next call) ->
 * dgpu_halo_stage_end (face term, lift, stage update and positivity). max_rhs (stage 2 only, may be NULL) is this
 * rank's max |rhs|, read after a stream synchronisation; reduce it over the ranks when needed. The residual alone:
 * dgpu_halo_rhs_begin / dgpu_halo_rhs_end, on the uploaded state. Euler and advection, QUAD/HEX. On a partitioned
 * context the whole-mesh entry points (dgpu_compute_rhs[_host], dgpu_ssp_rk3_step[s|_host], the Jacobian, JVP and
 * adjoint calls) return DGPU_ERR_INVALID_ARGUMENT. */
#define DGPU_REMOTE_VOLUME (-2)
dgpu_status dgpu_halo_setup(dgpu_ctx* ctx, int n_slots, const int* send_slots, const int* recv_slots);
dgpu_status dgpu_halo_buffers(dgpu_ctx* ctx, double** d_send, double** d_recv, size_t* slot_doubles);
dgpu_status dgpu_get_stream(dgpu_ctx* ctx, void** cuda_stream);
dgpu_status dgpu_halo_rhs_begin(dgpu_ctx* ctx);
dgpu_status dgpu_halo_rhs_end(dgpu_ctx* ctx, double* max_rhs);
dgpu_status dgpu_halo_stage_begin(dgpu_ctx* ctx, int stage);
dgpu_status dgpu_halo_stage_end(dgpu_ctx* ctx, double dt, int stage, double* max_rhs);
/* Measured FP64 FMA throughput of the current device in TFLOP/s (8 independent chains per thread, `iters`
 * iterations): the denominator of the FP64-pipe roofline. Measurement aid; no reference counterpart. */
dgpu_status dgpu_probe_fp64(int iters, double* tflops);
/* Measured FP64 tensor-core throughput (mma.sync m8n8k4 f64, 8 independent accumulators per warp) in TFLOP/s:
 * the evidence for or against routing the small contractions through DMMA. Measurement aid; no reference
 * counterpart. */
dgpu_status dgpu_probe_fp64_mma(int iters, double* tflops);
const char* dgpu_status_string(dgpu_status st);

/* ---- Batched residual over a mixed-order mesh ------------------------------------------------------------------
 * One context for a mesh whose volumes belong to several (element type, p) groups: QUAD (d = 2) or HEX (d = 3),
 * p = 1..4, one group per p. Advection, Euler, and Navier-Stokes (BR2, as dgpu_create; QUAD/HEX groups only, in
 * forms 0 and 2 below: the other forms and dense groups return DGPU_ERR_UNSUPPORTED). Replaces the same reference entry points as the uniform context above
 * (compute_rhs_dg, solve_dg.c:130-136; time_step_ssp_rk_33, solve_explicit.c:252-301) for a mesh with p
 * adaptation, where the reference's element loops visit volumes of different operator sets
 * (get_operator__cv0_vs_vc_T ... indexed by p, compute_volume_rlhs_dg_T.c) and integrates each face with the
 * cubature of order p_f = max(p_L, p_R) (face_solver.c:123-132).
 *
 *   ops[g]            the TP operator set of group g (distinct p per group)
 *   vol_group[v]      group of volume v
 *   mesh              as for dgpu_create with ragged blocks: volume v holds n_vc(v) = q(v)^d nodes, face f
 *                     holds n_fc(f) = q_f^(d-1) nodes with q_f = max(q(L), q(R)) (q(L) on a boundary face);
 *                     every array concatenates the blocks in list order. nc_fc (NULL: the identity) is, per
 *                     interior face, the reference's right-trace gather permutation at the face's q_f nodes
 *                     (get_operator__nc_fc_T(1, face), compute_face_rlhs_T.c:133-146): side 1's trace is read
 *                     at nc_fc[i] for side 0's node i, and side 1's lift reads the face flux through the
 *                     inverse; every side then writes its traces in its own face-node order (QUAD/HEX frames
 *                     may differ between neighbours). Boundary faces take bc_fc / bc_state_fc / bc_data as for dgpu_create
 *                     (Euler: BC_RIEMANN .. BC_SUPERSONIC_OUT; advection: the upwind codes).
 *
 * The state is the volumes' (n_vs(v) x n_var) column-major sol_coef blocks concatenated in volume-list order.
 * On the device the volumes are stored group by group; uploads and downloads permute. Each RK stage runs in one
 * of four forms: one launch per group for the volume and lift kernels and one per face order for the face kernel,
 * in sequence (form 0); one persistent launch each over a tile list that covers every group (form 1); the
 * launches of form 0 on parallel branches, so that the groups' kernels run concurrently (form 2); or the whole
 * stage as one cooperative persistent launch, its volume, face and lift phases separated by grid barriers
 * (form 3; a barrier that waits more than 2 s gives up and the call returns DGPU_ERR_CUDA). A step is
 * replayed from a captured CUDA graph in every form. No reference counterpart for the forms, the tile size or the
 * autotuner. */
typedef struct dgpu_batch dgpu_batch;
dgpu_status dgpu_batch_create(const dgpu_physics* phys, int n_groups, const dgpu_tp_operators* ops,
                              const int* vol_group, const dgpu_mesh* mesh, dgpu_batch** out);

/* Dense operator set of one non-tensor-product (TET, WEDGE or PYR, p) group: the reference's op_std operators
 * (cv0_vs_vc, cv1_vs_vc, cv0_vs_fc: element_operators.c; applied per volume by operator_T.c:96-156) for any
 * solution basis and cubature the caller uses. Row-major. M^-1 is constructor_mass_T's (volume_solver_T.c:115-145):
 * (cv0^T diag(w_vc) cv0)^-1 / J for an affine volume (constant jacobian_det_vc); in a group with a curved volume
 * (J varying over its nodes) every volume keeps its own (cv0^T diag(w_vc J_vc) cv0)^-1, formed on the device at
 * creation (n_vs^2 doubles per volume).
 * Face operators are evaluated at the face's canonical nodes (the node order the face's other side and the face
 * geometry use) as seen from local face lf under orientation ord (the reference's ind_ord, face.h:47-97):
 *   cv0_vs_fc[(lf * n_ord + ord) * 5 + p_f]   n_fc x n_vs, NULL where not provided;
 *   n_fc     [(lf * n_ord + ord) * 5 + p_f]   its number of face nodes (both sides of a face must agree);
 *   w_fc     [lf * 5 + p_f]                   the face cubature weights at the canonical nodes. */
typedef struct {
	int elem_type;                    /* DGPU_TRI (d = 2), DGPU_TET, DGPU_WEDGE or DGPU_PYR (d = 3) */
	int p;                            /* 1..4                                                      */
	int n_vs, n_vc;
	const double* cv0_vs_vc;          /* n_vc x n_vs                                               */
	const double* cv1_vs_vc;          /* d x n_vc x n_vs: d/dr_k of the basis at the vc nodes      */
	const double* w_vc;               /* n_vc                                                      */
	int n_lf;                         /* local faces: TET 4, WEDGE 5, PYR 5 (element.c f_ve order) */
	int n_ord;                        /* orientations per face (at most 8)                         */
	const int* n_fc;
	const double* const* cv0_vs_fc;
	const double* const* w_fc;
	/* Optional (WEDGE; NULL / 0 otherwise): the TRI x LINE factors of the volume operators, applied sum-factorised
	 * (the reference keeps such factors in Operator::ops_tp, operator.h:40-44): with basis index c * n_tri_vs + t
	 * and node index rz * n_tri_vc + rt, cv0_vs_vc = line_cv0 (x) tri_cv0, cv1_vs_vc[0/1] = line_cv0 (x)
	 * tri_cv1[0/1], cv1_vs_vc[2] = line_cv1 (x) tri_cv0. Checked against the dense operators at creation. */
	int n_tri_vs, n_tri_vc, n_line_vs, n_line_vc;
	const double* tri_cv0;            /* n_tri_vc x n_tri_vs                                       */
	const double* tri_cv1;            /* 2 x n_tri_vc x n_tri_vs                                   */
	const double* line_cv0;           /* n_line_vc x n_line_vs                                     */
	const double* line_cv1;           /* n_line_vc x n_line_vs                                     */
	/* Needed with positivity (NULL otherwise): solution-basis <-> Bezier coefficients, n_vs x n_vs row-major each
	 * (the element's ccSB0_vs_vs / ccBS0_vs_vs of enforce_positivity_highorder, solve.c:187-233). */
	const double* ccSB0_vs_vs;
	const double* ccBS0_vs_vs;
} dgpu_dense_operators;

/* One (type, p) group of a batched mesh: exactly one of tp / dense. */
typedef struct {
	const dgpu_tp_operators* tp;
	const dgpu_dense_operators* dense;
} dgpu_group;

/* Batched context over TP and dense groups. face_ord (n_faces x 2, may be NULL = all 0) gives each side's
 * orientation index into its face operator table; QUAD/HEX sides must have orientation 0. Two ways to describe a
 * face's nodes: a canonical order that each side's orientation-specific operators produce (face_ord, nc_fc NULL),
 * or the reference's own: every side's operators in its own face-node order (n_ord = 1, face_ord NULL) and the
 * face's data in side 0's order, with nc_fc (above) relating the sides. With positivity every dense group must
 * give its Bezier maps. */
dgpu_status dgpu_batch_create_groups(const dgpu_physics* phys, int n_groups, const dgpu_group* groups,
                                     const int* vol_group, const dgpu_mesh* mesh, const int* face_ord,
                                     dgpu_batch** out);
dgpu_status dgpu_batch_destroy(dgpu_batch* b);
/* Text of the last error of b (of the last failed dgpu_batch_create when b is NULL). */
const char* dgpu_batch_last_error(const dgpu_batch* b);
dgpu_status dgpu_batch_state_size(const dgpu_batch* b, size_t* n_doubles);
dgpu_status dgpu_batch_upload_state(dgpu_batch* b, const double* sol);   /* host, list order; synchronous */
/* The test case's source term, as dgpu_set_source: source_vc host, per volume (n_vc(v) x n_var) column-major, the
 * source at the volume cubature nodes before the J scaling, concatenated in volume-list order (n_vc of a dense
 * volume is its cubature node count); NULL removes it. The reference adds tw0_vt_vc (J s) to the rhs before M^-1
 * (compute_source_rhs_dg_like, src/simulation/solvers/compute_rlhs.c:47-57): a TP volume adds s to its GL nodal
 * residual after 1/(w J) (M^-1 tw0_vt_vc (J s) = V^-1 s); a TRI/TET/WEDGE/PYR volume's cv0^T diag(w J) s is formed
 * once here, on the host, and added before its M^-1. Every later residual and RK stage includes it, in every form. */
dgpu_status dgpu_batch_set_source(dgpu_batch* b, const double* source_vc);
dgpu_status dgpu_batch_download_state(dgpu_batch* b, double* sol);
dgpu_status dgpu_batch_download_rhs(dgpu_batch* b, double* rhs);
/* compute_rhs_dg on the device state; max_rhs as for dgpu_compute_rhs. */
dgpu_status dgpu_batch_compute_rhs(dgpu_batch* b, double* max_rhs);
/* n_steps SSP-RK3 steps (positivity included), graph-replayed. */
dgpu_status dgpu_batch_ssp_rk3_steps(dgpu_batch* b, double dt, int n_steps, double* max_rhs);
/* Form of the stages: 0 = one launch per group / face order in sequence, 1 = fused persistent launches,
 * 2 = the launches of form 0 on parallel branches, 3 = one cooperative persistent launch per stage. */
dgpu_status dgpu_batch_set_mode(dgpu_batch* b, int form);
/* Bound of each grid-barrier wait of form 3, in seconds (0 < seconds <= 60; 2 by default). A wait that runs out
 * ends the stage kernel and the call returns DGPU_ERR_CUDA; the context stays usable. */
dgpu_status dgpu_batch_set_barrier_timeout(dgpu_batch* b, double seconds);
dgpu_status dgpu_batch_get_mode(const dgpu_batch* b, int* form);
/* 1 (default): RK steps replay a captured CUDA graph; 0: every kernel is launched from the host each step. */
dgpu_status dgpu_batch_set_graphs(dgpu_batch* b, int enable);
/* Elements per CTA of group g in form 0 (1 .. 256 / q^d). */
dgpu_status dgpu_batch_set_group_tile(dgpu_batch* b, int group, int elements_per_cta);
/* Times every group's volume + lift kernels for each elements-per-CTA candidate (256/q^d, halved down to 1)
 * and keeps the fastest, then times `reps` RK steps of size dt in each of the four forms and keeps the
 * fastest. The device state is restored afterwards. A text report of the timings goes to `report`
 * (may be NULL). */
dgpu_status dgpu_batch_autotune(dgpu_batch* b, double dt, int reps, char* report, size_t report_len);
dgpu_status dgpu_batch_kernel_launches(const dgpu_batch* b, long long* n);
dgpu_status dgpu_batch_set_stream(dgpu_batch* b, void* cuda_stream);
dgpu_status dgpu_batch_positivity_corrections(dgpu_batch* b, long long* n);

#ifdef __cplusplus
}
#endif
#endif /* DGPU_H */
