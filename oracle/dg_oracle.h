/* CPU oracle for the explicit DG residual path (TEST INFRASTRUCTURE ONLY; see dg_oracle.c). */
#ifndef DG_ORACLE_H
#define DG_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
	ORACLE_OK = 0,
	ORACLE_ERR_ARG = -1,
	ORACLE_ERR_SINGULAR = -2,
	ORACLE_ERR_POSITIVITY = -3,
};

/* face_vol entry of a face side whose volume belongs to another partition of the mesh */
#define ORACLE_REMOTE_VOLUME (-2)

enum { ORACLE_PDE_ADVECTION = 1, ORACLE_PDE_EULER = 3, ORACLE_PDE_NAVIER_STOKES = 4 };   /* definitions_test_case.h */
enum { ORACLE_VISCOSITY_CONSTANT = 101, ORACLE_VISCOSITY_SUTHERLAND = 102 };  /* definitions_physics.h:34-36 */
enum { ORACLE_NUM_FLUX_UPWIND = 11, ORACLE_NUM_FLUX_ROE_PIKE = 31, ORACLE_NUM_FLUX_LAX_FRIEDRICHS = 32 };

/* One (element type, p): the reference's dense (op_std) volume operators. Row-major. */
struct oracle_group {
	int n_vs, n_vc;
	const double* cv0_vs_vc;   /* n_vc x n_vs */
	const double* tw1_vt_vc;   /* d x (n_vs x n_vc) */
	const double* w_vc;        /* n_vc */
	const double* ccSB0;       /* n_vs x n_vs  Lagrange -> Bezier coefficients */
	const double* ccBS0;       /* n_vs x n_vs  Bezier -> Lagrange coefficients */
	const double* cv1_vs_vc;   /* d x (n_vc x n_vs): basis derivatives at the volume cubature nodes (Navier-Stokes) */
};

/* Face operators of a volume of one group at one face cubature order p_f (cv0_vs_fc[lf][p_f][p_v],
 * tw0_vt_fc likewise: compute_face_rlhs_T.c:51-81). Row-major. */
struct oracle_face_ops {
	int n_fc, n_vs;
	const double* cv0_vs_fc;   /* 2d x (n_fc x n_vs) */
	const double* tw0_vt_fc;   /* 2d x (n_vs x n_fc) */
};

/* A mesh of volumes of any number of groups. States and per-volume node arrays are concatenated in volume-list
 * order (per volume the reference's column-major blocks); per-face arrays in face-list order. The oracle keeps
 * pointers to these arrays: they must outlive the context. */
struct oracle_problem {
	int d, n_var, pde, num_flux, positivity;
	double b_adv[3];
	int n_groups;
	const struct oracle_group* groups;
	int n_face_ops;
	const struct oracle_face_ops* face_ops;
	int n_volumes;
	const int* vol_group;
	const double* metrics_vc;      /* per volume (n_vc, d, d) column-major */
	const double* jacobian_det_vc; /* per volume n_vc */
	int n_faces;
	const int* face_vol;           /* n_faces x 2 */
	const int* face_lf;            /* n_faces x 2 */
	const int* face_ops_idx;       /* n_faces x 2: face operator set of each side */
	const int* nc_fc;              /* per face n_fc: right trace gathered as sR[i] = sR_own[nc_fc[i]] */
	const double* normals_fc;      /* per face (n_fc x d) row-major */
	const double* jacobian_det_fc; /* per face n_fc */
	/* Boundary faces have face_vol[2f+1] < 0. bc_fc: per face the reference's BC code (definitions_bc.h; 0 or any
	 * value on interior faces); bc_state_fc: per face (n_fc x n_var) row-major exterior conserved state
	 * (constructor_sol_bv at the face nodes). Both may be NULL on meshes without boundary faces. */
	const int* bc_fc;
	const double* bc_state_fc;
	/* BC_Data of boundary_euler_T.c:44-49, read from the test case's input by the reference: p_back (BC_BACKPRESSURE
	 * 103), t_total, p_total, r_s (BC_TOTAL_TP 104). */
	double bc_data[4];
	/* Navier-Stokes (pde 4): viscosity model (VISCOSITY_CONSTANT 101 / VISCOSITY_SUTHERLAND 102), mu (the constant
	 * viscosity, or the reference value Sutherland's law scales), Prandtl number, specific gas constant (Sutherland's
	 * temperature), read from the test case's input by the reference (solution_navier_stokes_T.c:188-255,
	 * flux_navier_stokes_T.c:461-482). The second-order numerical flux is BR2 (NUM_FLUX_BR2_STABLE), the only
	 * explicit option the reference's DG solver provides. */
	int viscosity;
	double mu, Pr, r_s;
	/* BC_NOSLIP_DIABATIC 112: the wall's normal temperature gradient dTdn (diabatic_flux_type constant; 0 for
	 * constant_zero), which sets the wall's normal energy flux nf_E = -mu Cp / Pr dTdn (get_normal_flux_Energy,
	 * solution_navier_stokes.c:93-150). */
	double dTdn;
	/* Source term of the test case: per volume (n_vc x n_var) column-major, the source at the volume cubature nodes
	 * before the J scaling (what constructor_source_* returns), or NULL. compute_source_rhs_dg_like
	 * (compute_rlhs.c:47-57) adds tw0_vt_vc (J_vc s) to each volume's rhs
	 * (compute_source_rhs_advection_default_T, solution_advection_default_T.c:79-94). */
	const double* source_vc;
};

struct oracle_ctx;

int oracle_create(const struct oracle_problem* in, struct oracle_ctx** out);
void oracle_destroy(struct oracle_ctx* c);
size_t oracle_state_size(const struct oracle_ctx* c);
int oracle_compute_rhs(const struct oracle_ctx* c, const double* sol, double* rhs, double* max_rhs);
int oracle_compute_rhs_raw(const struct oracle_ctx* c, const double* sol, double* rhs);
int oracle_compute_rhs_cmplx(const struct oracle_ctx* c, const double* sol_re, const double* sol_im,
                             double* rhs_re, double* rhs_im);
int oracle_ssp_rk3_step(const struct oracle_ctx* c, double dt, double* sol, double* max_rhs, int* n_corrections);
int oracle_face_traces(const struct oracle_ctx* c, const double* sol, int n, const int* slots, double* out);
int oracle_compute_rhs_remote(const struct oracle_ctx* c, const double* sol, const double* remote, double* rhs,
                              double* max_rhs);
size_t oracle_face_node_total(const struct oracle_ctx* c);
int oracle_enforce_positivity(const struct oracle_ctx* c, double* sol, int* n_corrections);
/* M^-1 of volume v (n_vs x n_vs row-major) */
const double* oracle_m_inv(const struct oracle_ctx* c, int v);

#ifdef __cplusplus
}
#endif
#endif
