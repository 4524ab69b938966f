/* CPU oracle for the explicit DG residual path of DPGSolver.
 *
 * TEST INFRASTRUCTURE ONLY. This plain-C restatement of the reference's algorithm is the checker that the
 * CUDA path is compared against; only tests, the smoke check and the CPU-baseline leg of the benchmark load
 * it. Nothing in the product links or calls it.
 *
 * It follows the reference's own data flow with dense ("op_std", op_format 'd') operators, element by
 * element, in volume-list and face-list order:
 *   compute_rhs_dg            src/simulation/solvers/dg/solve_dg.c:130-136
 *   compute_rlhs_common_dg    src/simulation/solvers/dg/solve_dg.c:182-189
 *   scale_rhs_by_m_inv_std    src/simulation/solvers/dg/solve_dg.c:265-272
 *   compute_max_rhs_dg_like   src/simulation/solvers/compute_rlhs.c:59-71
 *   time_step_ssp_rk_33       src/simulation/solvers/solve_explicit.c:252-301
 *   enforce_positivity_highorder  src/simulation/solvers/solve.c:187-233, correct_coef :356-374
 *   constructor_mass_T / constructor_inverse_mass_T  src/simulation/solvers/volume_solver_T.c:115-145
 * The double instantiation gives the residual and the time step; the double complex instantiation gives the
 * complex-step linearisation the reference uses in test_support_solve_dg.c:83-110.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "dg_oracle.h"

#define GAMMA 1.4          /* definitions_physics.h:23 */
#define GM1 0.4            /* definitions_physics.h:24 */
#define EPS_PHYS 1.0e-13   /* definitions_physics.h:30 */
#define ORACLE_EPS 1.0e-15 /* definitions_tol.h:23 */

struct oracle_ctx {
	struct oracle_problem P;       /* pointers into the caller's arrays (they must outlive the context) */
	size_t n_state;
	size_t *state_off, *vc_off, *fc_off, *minv_off;   /* per volume / per face offsets */
	int max_vs, max_vc, max_fc;
	double* m_inv;                 /* per volume n_vs x n_vs row-major */
};

/* ---- double instantiation ---- */
#define Type double
#define SUF(name) name##_d
#define REAL_T(x) (x)
#define ABS_T(x) fabs(x)
#define SQRT_T(x) sqrt(x)
#define POW_T(x, y) pow(x, y)
#include "dg_oracle_T.h"
#undef Type
#undef SUF
#undef REAL_T
#undef ABS_T
#undef SQRT_T
#undef POW_T

/* ---- double complex instantiation ---- */
#define Type double complex
#define SUF(name) name##_c
#define REAL_T(x) creal(x)
#define ABS_T(x) cabs(x)
#define SQRT_T(x) csqrt(x)
#define POW_T(x, y) cpow(x, y)
#include "dg_oracle_T.h"
#undef Type
#undef SUF
#undef REAL_T
#undef ABS_T
#undef SQRT_T
#undef POW_T

/* Inverse by Gauss-Jordan elimination with partial pivoting (the reference solves with the identity as
 * right-hand side through LAPACKE, matrix_constructors_T.c constructor_inverse_const_Matrix_T). */
static int invert(const int n, const double* A, double* Ainv)
{
	double* a = malloc(sizeof(double) * (size_t)n * n);
	memcpy(a, A, sizeof(double) * (size_t)n * n);
	for (int i = 0; i < n; ++i)
		for (int j = 0; j < n; ++j)
			Ainv[i * n + j] = (i == j ? 1.0 : 0.0);
	for (int col = 0; col < n; ++col) {
		int piv = col;
		for (int r = col + 1; r < n; ++r)
			if (fabs(a[r * n + col]) > fabs(a[piv * n + col]))
				piv = r;
		if (a[piv * n + col] == 0.0) {
			free(a);
			return ORACLE_ERR_SINGULAR;
		}
		if (piv != col) {
			for (int j = 0; j < n; ++j) {
				double t = a[col * n + j]; a[col * n + j] = a[piv * n + j]; a[piv * n + j] = t;
				t = Ainv[col * n + j]; Ainv[col * n + j] = Ainv[piv * n + j]; Ainv[piv * n + j] = t;
			}
		}
		const double inv = 1.0 / a[col * n + col];
		for (int j = 0; j < n; ++j) {
			a[col * n + j] *= inv;
			Ainv[col * n + j] *= inv;
		}
		for (int r = 0; r < n; ++r) {
			if (r == col)
				continue;
			const double fct = a[r * n + col];
			if (fct == 0.0)
				continue;
			for (int j = 0; j < n; ++j) {
				a[r * n + j] -= fct * a[col * n + j];
				Ainv[r * n + j] -= fct * Ainv[col * n + j];
			}
		}
	}
	free(a);
	return ORACLE_OK;
}

int oracle_create(const struct oracle_problem* in, struct oracle_ctx** out)
{
	if (!in || !out)
		return ORACLE_ERR_ARG;
	if (in->d < 2 || in->d > 3 || in->n_volumes < 1 || in->n_groups < 1 || in->n_face_ops < 1)
		return ORACLE_ERR_ARG;
	if ((in->pde == ORACLE_PDE_EULER || in->pde == ORACLE_PDE_NAVIER_STOKES) && in->n_var != in->d + 2)
		return ORACLE_ERR_ARG;
	if (in->pde == ORACLE_PDE_ADVECTION && in->n_var != 1)
		return ORACLE_ERR_ARG;
	if (in->pde == ORACLE_PDE_NAVIER_STOKES) {   /* gradients need the basis derivatives; no boundary values yet */
		if ((in->viscosity != ORACLE_VISCOSITY_CONSTANT && in->viscosity != ORACLE_VISCOSITY_SUTHERLAND) ||
		    !(in->Pr > 0.0) || !(in->mu >= 0.0))
			return ORACLE_ERR_ARG;
		/* a non-zero wall heat flux needs constant viscosity (the assertion of get_normal_flux_Energy) */
		if (in->dTdn != 0.0 && in->viscosity != ORACLE_VISCOSITY_CONSTANT)
			return ORACLE_ERR_ARG;
		for (int g = 0; g < in->n_groups; ++g)
			if (!in->groups[g].cv1_vs_vc)
				return ORACLE_ERR_ARG;
	}
	if (in->positivity)   /* the limiter needs every group's Bezier maps */
		for (int g = 0; g < in->n_groups; ++g)
			if (!in->groups[g].ccSB0 || !in->groups[g].ccBS0)
				return ORACLE_ERR_ARG;
	struct oracle_ctx* c = calloc(1, sizeof *c);
	c->P = *in;
	const int d = in->d, nv = in->n_var;
	const size_t nV = (size_t)in->n_volumes, nF = (size_t)in->n_faces;
	c->state_off = malloc(sizeof(size_t) * (nV + 1));
	c->vc_off = malloc(sizeof(size_t) * (nV + 1));
	c->minv_off = malloc(sizeof(size_t) * (nV + 1));
	c->fc_off = malloc(sizeof(size_t) * (nF + 1));
	size_t so = 0, vo = 0, mo = 0, fo = 0;
	for (size_t v = 0; v < nV; ++v) {
		const int g = in->vol_group[v];
		if (g < 0 || g >= in->n_groups) {
			oracle_destroy(c);
			return ORACLE_ERR_ARG;
		}
		const struct oracle_group* G = &in->groups[g];
		c->state_off[v] = so;
		c->vc_off[v] = vo;
		c->minv_off[v] = mo;
		so += (size_t)G->n_vs * nv;
		vo += (size_t)G->n_vc;
		mo += (size_t)G->n_vs * G->n_vs;
		if (G->n_vs > c->max_vs) c->max_vs = G->n_vs;
		if (G->n_vc > c->max_vc) c->max_vc = G->n_vc;
	}
	c->state_off[nV] = so;
	c->n_state = so;
	for (size_t f = 0; f < nF; ++f) {
		const struct oracle_face_ops* FL = &in->face_ops[in->face_ops_idx[2 * f]];
		const struct oracle_face_ops* FR = &in->face_ops[in->face_ops_idx[2 * f + 1]];
		const int rem0 = in->face_vol[2 * f] == ORACLE_REMOTE_VOLUME, rem1 = in->face_vol[2 * f + 1] == ORACLE_REMOTE_VOLUME;
		const int boundary = in->face_vol[2 * f + 1] < 0 && !rem1;
		if ((!boundary && FL->n_fc != FR->n_fc) || (boundary && (!in->bc_fc || !in->bc_state_fc)) || (rem0 && rem1) ||
		    (!rem0 && (in->face_vol[2 * f] < 0 || in->face_vol[2 * f] >= in->n_volumes))) {
			oracle_destroy(c);
			return ORACLE_ERR_ARG;
		}
		c->fc_off[f] = fo;
		fo += (size_t)FL->n_fc;
		if (FL->n_fc > c->max_fc) c->max_fc = FL->n_fc;
	}
	c->fc_off[nF] = fo;
	(void)d;

	/* M = cv0_vs_vc^T diag(w_vc J_vc) cv0_vs_vc, m_inv = M^-1 (volume_solver_T.c:115-145). A volume whose J is the
	 * same at every cubature node (an affine volume) has M = J M_ref: its inverse is the group's M_ref^-1 / J, formed
	 * once per group (equal to inverting J M_ref up to rounding). */
	c->m_inv = malloc(sizeof(double) * (mo ? mo : 1));
	double* M = malloc(sizeof(double) * (size_t)c->max_vs * c->max_vs);
	double** ref_inv = calloc((size_t)in->n_groups, sizeof(double*));
	for (size_t v = 0; v < nV; ++v) {
		const int g = in->vol_group[v];
		const struct oracle_group* G = &in->groups[g];
		const int n_vs = G->n_vs, n_vc = G->n_vc;
		const double* J = &in->jacobian_det_vc[c->vc_off[v]];
		int affine = 1;
		for (int k = 1; k < n_vc && affine; ++k)
			affine = (J[k] == J[0]);
		if (affine) {
			if (!ref_inv[g]) {
				for (int i = 0; i < n_vs; ++i)
					for (int j = 0; j < n_vs; ++j) {
						double s = 0.0;
						for (int k = 0; k < n_vc; ++k)
							s += G->cv0_vs_vc[k * n_vs + i] * G->w_vc[k] * G->cv0_vs_vc[k * n_vs + j];
						M[i * n_vs + j] = s;
					}
				ref_inv[g] = malloc(sizeof(double) * (size_t)n_vs * n_vs);
				const int st = invert(n_vs, M, ref_inv[g]);
				if (st != ORACLE_OK) {
					for (int k = 0; k < in->n_groups; ++k)
						free(ref_inv[k]);
					free(ref_inv);
					free(M);
					oracle_destroy(c);
					return st;
				}
			}
			double* Mi = &c->m_inv[c->minv_off[v]];
			for (int i = 0; i < n_vs * n_vs; ++i)
				Mi[i] = ref_inv[g][i] / J[0];
			continue;
		}
		for (int i = 0; i < n_vs; ++i)
			for (int j = 0; j < n_vs; ++j) {
				double s = 0.0;
				for (int k = 0; k < n_vc; ++k)
					s += G->cv0_vs_vc[k * n_vs + i] * (G->w_vc[k] * J[k]) * G->cv0_vs_vc[k * n_vs + j];
				M[i * n_vs + j] = s;
			}
		int st = invert(n_vs, M, &c->m_inv[c->minv_off[v]]);
		if (st != ORACLE_OK) {
			for (int k = 0; k < in->n_groups; ++k)
				free(ref_inv[k]);
			free(ref_inv);
			free(M);
			oracle_destroy(c);
			return st;
		}
	}
	free(M);
	for (int k = 0; k < in->n_groups; ++k)
		free(ref_inv[k]);
	free(ref_inv);
	*out = c;
	return ORACLE_OK;
}

void oracle_destroy(struct oracle_ctx* c)
{
	if (!c)
		return;
	free(c->m_inv);
	free(c->state_off);
	free(c->vc_off);
	free(c->minv_off);
	free(c->fc_off);
	free(c);
}

size_t oracle_state_size(const struct oracle_ctx* c)
{
	return c->n_state;
}

int oracle_compute_rhs(const struct oracle_ctx* c, const double* sol, double* rhs, double* max_rhs)
{
	int st = residual_raw_d(c, sol, rhs, NULL);
	if (st != ORACLE_OK)
		return st;
	scale_m_inv_d(c, rhs);
	double mx = 0.0;
	const size_t n = oracle_state_size(c);
	for (size_t i = 0; i < n; ++i)
		if (fabs(rhs[i]) > mx)
			mx = fabs(rhs[i]);
	if (max_rhs)
		*max_rhs = mx;
	return ORACLE_OK;
}

int oracle_compute_rhs_raw(const struct oracle_ctx* c, const double* sol, double* rhs)
{
	return residual_raw_d(c, sol, rhs, NULL);
}

/* Partitioned meshes: the traces of the given face sides (slot 2f+s, a side with a volume of this mesh), each
 * n_fc x n_var column-major in the side's own face-node order (cv0_vs_fc[ind_lf] s_coef, compute_face_rlhs_T.c:67-81),
 * at out + i * n_fc * n_var. */
int oracle_face_traces(const struct oracle_ctx* c, const double* sol, int n, const int* slots, double* out)
{
	const struct oracle_problem* P = &c->P;
	const int nv = P->n_var;
	size_t o = 0;
	for (int i = 0; i < n; ++i) {
		const int f = slots[i] / 2, s = slots[i] % 2;
		if (slots[i] < 0 || f >= P->n_faces)
			return ORACLE_ERR_ARG;
		const int v = P->face_vol[2 * f + s], lf = P->face_lf[2 * f + s];
		if (v < 0 || v >= P->n_volumes)
			return ORACLE_ERR_ARG;
		const struct oracle_face_ops* F = &P->face_ops[P->face_ops_idx[2 * f + s]];
		for (size_t k = 0; k < (size_t)F->n_fc * nv; ++k)
			out[o + k] = 0.0;
		mm_acc_d(F->n_fc, F->n_vs, nv, 1.0, &F->cv0_vs_fc[(size_t)lf * F->n_fc * F->n_vs], &sol[c->state_off[v]],
		         &out[o]);
		o += (size_t)F->n_fc * nv;
	}
	return ORACLE_OK;
}

/* oracle_compute_rhs on a partition: remote holds, per face, the trace of its side that belongs to another
 * partition (face_vol == ORACLE_REMOTE_VOLUME), n_fc x n_var column-major at fc_off[f] * n_var. */
int oracle_compute_rhs_remote(const struct oracle_ctx* c, const double* sol, const double* remote, double* rhs,
                              double* max_rhs)
{
	int st = residual_raw_d(c, sol, rhs, remote);
	if (st != ORACLE_OK)
		return st;
	scale_m_inv_d(c, rhs);
	double mx = 0.0;
	const size_t n = oracle_state_size(c);
	for (size_t i = 0; i < n; ++i)
		if (fabs(rhs[i]) > mx)
			mx = fabs(rhs[i]);
	if (max_rhs)
		*max_rhs = mx;
	return ORACLE_OK;
}

size_t oracle_face_node_total(const struct oracle_ctx* c)
{
	return c->fc_off[c->P.n_faces];
}

int oracle_compute_rhs_cmplx(const struct oracle_ctx* c, const double* sol_re, const double* sol_im,
                             double* rhs_re, double* rhs_im)
{
	const size_t n = oracle_state_size(c);
	double complex* s = malloc(sizeof(double complex) * n);
	double complex* r = malloc(sizeof(double complex) * n);
	for (size_t i = 0; i < n; ++i)
		s[i] = sol_re[i] + I * (sol_im ? sol_im[i] : 0.0);
	int st = residual_raw_c(c, s, r, NULL);
	if (st == ORACLE_OK) {
		scale_m_inv_c(c, r);
		for (size_t i = 0; i < n; ++i) {
			rhs_re[i] = creal(r[i]);
			rhs_im[i] = cimag(r[i]);
		}
	}
	free(s);
	free(r);
	return st;
}

/* convert_variables_T (solution_euler_T.c:136-200) on one volume's (n_n x n_var) column-major block. */
static void convert_c_to_p(const int d, const int n_n, double* v)
{
	double* rho = &v[0];
	double* E = &v[(size_t)n_n * (d + 1)];
	for (int i = 0; i < n_n; ++i) {
		const double rho_inv = 1.0 / rho[i];
		double rho2V2 = 0.0;
		for (int k = 0; k < d; ++k) {
			double* m = &v[(size_t)n_n * (1 + k)];
			rho2V2 += m[i] * m[i];
			m[i] = m[i] * rho_inv;
		}
		E[i] = GM1 * (E[i] - 0.5 * rho2V2 * rho_inv);
	}
}

static void convert_p_to_c(const int d, const int n_n, double* v)
{
	double* rho = &v[0];
	double* p = &v[(size_t)n_n * (d + 1)];
	for (int i = 0; i < n_n; ++i) {
		double V2 = 0.0;
		for (int k = 0; k < d; ++k) {
			double* u = &v[(size_t)n_n * (1 + k)];
			V2 += u[i] * u[i];
			u[i] = rho[i] * u[i];
		}
		p[i] = p[i] / GM1 + 0.5 * rho[i] * V2;
	}
}

static double average(const double* a, int n)
{
	double s = 0.0;
	for (int i = 0; i < n; ++i)
		s += a[i];
	return s / n;
}

/* enforce_positivity_highorder (solve.c:187-233) for one volume. Returns 1 when correct_coef was applied
 * (for density, pressure or both), 0 when not, or a negative error. */
static int enforce_positivity(const struct oracle_ctx* c, int v, double* s_coef)
{
	const struct oracle_problem* P = &c->P;
	const struct oracle_group* G = &P->groups[P->vol_group[v]];
	const int n_n = G->n_vs, n_vr = P->n_var, d = P->d;
	double* sb = calloc((size_t)n_n * n_vr, sizeof(double));
	mm_acc_d(n_n, n_n, n_vr, 1.0, G->ccSB0, s_coef, sb);
	convert_c_to_p(d, n_n, sb);
	int n_corr = 0;
	for (int vr = 0; vr < n_vr; vr += n_vr - 1) {
		double* vd = &sb[(size_t)vr * n_n];
		const double vr_avg = average(vd, n_n);
		if (vr_avg < EPS_PHYS) {
			free(sb);
			return ORACLE_ERR_POSITIVITY;
		}
		double vr_min = vd[0];
		for (int i = 1; i < n_n; ++i)
			if (vd[i] < vr_min)
				vr_min = vd[i];
		if (vr_min < EPS_PHYS) {
			double p_ho = (vr_avg - EPS_PHYS) / (vr_avg - vr_min);
			p_ho = fmax(0.0, fmin(1.0, p_ho));
			/* correct_coef (solve.c:356-374) */
			for (int w = 0; w < n_vr; ++w) {
				double* data = &sb[(size_t)w * n_n];
				double avg = average(data, n_n);
				if ((w == 0 || w == n_vr - 1) && avg < EPS_PHYS)
					avg = EPS_PHYS;
				for (int i = 0; i < n_n; ++i)
					data[i] = p_ho * data[i] + (1 - p_ho) * avg;
			}
			n_corr = 1;
		}
		if (n_vr == 1)
			break;
	}
	convert_p_to_c(d, n_n, sb);
	for (size_t i = 0; i < (size_t)n_n * n_vr; ++i)
		s_coef[i] = 0.0;
	mm_acc_d(n_n, n_n, n_vr, 1.0, G->ccBS0, sb, s_coef);
	free(sb);
	return n_corr;
}

int oracle_ssp_rk3_step(const struct oracle_ctx* c, const double dt, double* sol, double* max_rhs,
                        int* n_corrections)
{
	const struct oracle_problem* P = &c->P;
	const size_t n = oracle_state_size(c);
	double* rhs = malloc(sizeof(double) * n);
	double* sp = malloc(sizeof(double) * n);
	double mx = 0.0;
	int ncorr = 0;
	int st = ORACLE_OK;
	for (int rk = 0; rk < 3 && st == ORACLE_OK; ++rk) {
		st = oracle_compute_rhs(c, sol, rhs, &mx);
		if (st != ORACLE_OK)
			break;
		for (int v = 0; v < P->n_volumes; ++v) {
			const size_t o = c->state_off[v], vs_sz = c->state_off[v + 1] - o;
			double* s = &sol[o];
			double* p = &sp[o];
			const double* r = &rhs[o];
			switch (rk) {
			case 0:
				for (size_t i = 0; i < vs_sz; ++i) {
					p[i] = s[i];
					s[i] += dt * r[i];
				}
				break;
			case 1:
				for (size_t i = 0; i < vs_sz; ++i)
					s[i] = (1.0 / 4.0) * (3.0 * p[i] + s[i] + dt * r[i]);
				break;
			default:
				for (size_t i = 0; i < vs_sz; ++i)
					s[i] = (1.0 / 3.0) * (p[i] + 2.0 * s[i] + 2.0 * dt * r[i]);
				break;
			}
			if (P->positivity) {
				int k = enforce_positivity(c, v, s);
				if (k < 0) {
					st = k;
					break;
				}
				ncorr += k;
			}
		}
	}
	free(rhs);
	free(sp);
	if (max_rhs)
		*max_rhs = mx;
	if (n_corrections)
		*n_corrections = ncorr;
	return st;
}

int oracle_enforce_positivity(const struct oracle_ctx* c, double* sol, int* n_corrections)
{
	int ncorr = 0;
	for (int v = 0; v < c->P.n_volumes; ++v) {
		int k = enforce_positivity(c, v, &sol[c->state_off[v]]);
		if (k < 0)
			return k;
		ncorr += k;
	}
	if (n_corrections)
		*n_corrections = ncorr;
	return ORACLE_OK;
}

const double* oracle_m_inv(const struct oracle_ctx* c, int v)
{
	return &c->m_inv[c->minv_off[v]];
}
