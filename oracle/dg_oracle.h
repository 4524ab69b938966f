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

enum { ORACLE_PDE_ADVECTION = 1, ORACLE_PDE_EULER = 3 };                  /* definitions_test_case.h */
enum { ORACLE_NUM_FLUX_UPWIND = 11, ORACLE_NUM_FLUX_ROE_PIKE = 31, ORACLE_NUM_FLUX_LAX_FRIEDRICHS = 32 };

/* One (element type, p) group with dense reference operators; all volumes share it.
 * Operators row-major; states and per-volume node arrays column-major like the reference's 'C' Multiarrays. */
struct oracle_problem {
	int d, n_var, pde, num_flux, positivity;
	double b_adv[3];
	int n_vs, n_vc, n_fc;
	const double* cv0_vs_vc;   /* n_vc x n_vs */
	const double* tw1_vt_vc;   /* d x (n_vs x n_vc) */
	const double* cv0_vs_fc;   /* 2d x (n_fc x n_vs) */
	const double* tw0_vt_fc;   /* 2d x (n_vs x n_fc) */
	const double* w_vc;        /* n_vc */
	const double* ccSB0;       /* n_vs x n_vs  Lagrange -> Bezier coefficients */
	const double* ccBS0;       /* n_vs x n_vs  Bezier -> Lagrange coefficients */
	int n_volumes;
	const double* metrics_vc;      /* n_volumes x (n_vc, d, d) column-major */
	const double* jacobian_det_vc; /* n_volumes x n_vc */
	int n_faces;
	const int* face_vol;           /* n_faces x 2 */
	const int* face_lf;            /* n_faces x 2 */
	const int* nc_fc;              /* n_faces x n_fc: right trace gathered as sR[i] = sR_own[nc_fc[i]] */
	const double* normals_fc;      /* n_faces x (n_fc x d) row-major */
	const double* jacobian_det_fc; /* n_faces x n_fc */
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
int oracle_enforce_positivity(const struct oracle_ctx* c, double* sol, int* n_corrections);
const double* oracle_m_inv(const struct oracle_ctx* c);

#ifdef __cplusplus
}
#endif
#endif
