/* A C11 host program that calls the GB300 residual through include/dgpu.h the way DPGSolver's own C code would:
 * it holds the mesh as the reference does (intrusive lists of solver volumes and faces, each owning its multiarrays
 * in the reference's layouts), packs them once in list order (pack_from_sim, the set-up of INTEGRATION.md section
 * 1), and replaces the two entry points of the explicit solver:
 *     compute_rhs_dg       (src/simulation/solvers/dg/solve_dg.c:130-136)      -> dgpu_compute_rhs_host
 *     time_step_ssp_rk_33  (src/simulation/solvers/solve_explicit.c:252-301)   -> dgpu_ssp_rk3_step_host
 * each reading Solver_Volume::sol_coef and writing back Solver_Volume::rhs / sol_coef.
 *
 *     dgpu_caller <case.bin> <out.bin>
 *
 * case.bin (little endian, written by tests/test_gpu_c_caller.py):
 *   int32  magic 0x55504744, d, p, pde, num_flux, positivity, n_volumes, n_faces, n_steps
 *   f64    dt, b_adv[3]
 *   int32  viscosity; f64 mu, Pr, r_s, dTdn (Navier-Stokes constants of the test case's input; 0 otherwise)
 *   f64    bc_data[4] (p_back, t_total, p_total, r_s of the back-pressure / total T/p faces; 0 when none)
 *   f64    1D operators: cv0_vs_vc (q x q), cv1_vs_vc (q x q), cv0_vs_fc (2 x q), w_vc (q), ccSB0 (q x q), ccBS0 (q x q)
 *   per volume:  f64 metrics_vc (n_vc, d, d) 'C', jacobian_det_vc (n_vc), sol_coef (n_vs, n_var) 'C'
 *   per face:    int32 volume[2], ind_lf[2], ind_ord[2] (volume -1 on a boundary face's missing side), bc;
 *                f64 normals_fc (n_fc, d) 'R', jacobian_det_fc (n_fc); on a boundary face also the exterior state
 *                (n_fc, n_var) 'R' (constructor_sol_bv at its nodes, or the rotating wall's state)
 * out.bin: per volume rhs (n_vs, n_var) 'C' after compute_rhs_dg, then f64 max_rhs; per volume sol_coef after
 * n_steps calls of time_step_ssp_rk_33, then f64 max_rhs of the last step.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dgpu.h"

/* ------------------------------------------------------------------------------------------------------------
 * The reference's containers, reduced to what this path touches (multiarray.h, intrusive.h, volume_solver_T.h,
 * face_solver_T.h, face.h).
 * ------------------------------------------------------------------------------------------------------------ */
struct Multiarray_d {
	char layout;            /* 'C' column-major or 'R' row-major                   */
	int order;
	ptrdiff_t extents[3];
	double* data;
};

struct Intrusive_Link {
	struct Intrusive_Link* next;
};

struct Solver_Volume {
	struct Intrusive_Link lnk;   /* first member, as in the reference: a link is its volume */
	int index;
	struct Multiarray_d sol_coef, rhs, metrics_vc, jacobian_det_vc;
};

struct Neigh_Info {
	int ind_lf, ind_ord;
	struct Solver_Volume* volume;
};

struct Solver_Face {
	struct Intrusive_Link lnk;
	int index;
	int boundary, bc;                 /* Face::boundary, Face::bc */
	struct Neigh_Info neigh_info[2];
	struct Multiarray_d normals_fc, jacobian_det_fc;
	struct Multiarray_d s_bv;         /* the exterior state at the face nodes (boundary faces) */
};

struct Simulation {
	int d, p, pde, num_flux, positivity, n_var, n_vs, n_vc, n_fc, n_v, n_f;
	double b_adv[3];
	int viscosity;
	double mu, Pr, r_s, dTdn, bc_data[4];
	struct Intrusive_Link* volumes;   /* first link of each list */
	struct Intrusive_Link* faces;
};

static void die(const char* what)
{
	fprintf(stderr, "dgpu_caller: %s\n", what);
	exit(1);
}

static void ma_init(struct Multiarray_d* a, char layout, int order, ptrdiff_t e0, ptrdiff_t e1, ptrdiff_t e2)
{
	a->layout = layout;
	a->order = order;
	a->extents[0] = e0;
	a->extents[1] = e1;
	a->extents[2] = e2;
	size_t n = (size_t)e0 * (order > 1 ? (size_t)e1 : 1) * (order > 2 ? (size_t)e2 : 1);
	a->data = calloc(n ? n : 1, sizeof(double));
	if (!a->data)
		die("out of memory");
}

static size_t ma_size(const struct Multiarray_d* a)
{
	return (size_t)a->extents[0] * (a->order > 1 ? (size_t)a->extents[1] : 1) *
	       (a->order > 2 ? (size_t)a->extents[2] : 1);
}

static void rd(void* dst, size_t size, size_t n, FILE* f)
{
	if (fread(dst, size, n, f) != n)
		die("case file too short");
}

/* ------------------------------------------------------------------------------------------------------------
 * Reading the case into reference-shaped lists (what the reference's own set-up would have built).
 * ------------------------------------------------------------------------------------------------------------ */
struct Operators {
	double *cv0, *cv1, *cv0_fc, *w, *sb, *bs;
};

static void read_case(const char* path, struct Simulation* sim, struct Operators* ops, int* n_steps, double* dt)
{
	FILE* f = fopen(path, "rb");
	if (!f)
		die("cannot open the case file");
	int32_t h[9];
	rd(h, sizeof(int32_t), 9, f);
	if (h[0] != 0x55504744)
		die("bad magic");
	sim->d = h[1];
	sim->p = h[2];
	sim->pde = h[3];
	sim->num_flux = h[4];
	sim->positivity = h[5];
	sim->n_v = h[6];
	sim->n_f = h[7];
	*n_steps = h[8];
	rd(dt, sizeof(double), 1, f);
	rd(sim->b_adv, sizeof(double), 3, f);
	int32_t visc;
	double nsc[4];
	rd(&visc, sizeof(int32_t), 1, f);
	rd(nsc, sizeof(double), 4, f);
	rd(sim->bc_data, sizeof(double), 4, f);
	sim->viscosity = visc;
	sim->mu = nsc[0];
	sim->Pr = nsc[1];
	sim->r_s = nsc[2];
	sim->dTdn = nsc[3];
	const int q = sim->p + 1, d = sim->d;
	sim->n_var = (sim->pde == DGPU_PDE_ADVECTION ? 1 : d + 2);
	sim->n_vs = sim->n_vc = (d == 2 ? q * q : q * q * q);
	sim->n_fc = (d == 2 ? q : q * q);

	double** slots[6] = {&ops->cv0, &ops->cv1, &ops->cv0_fc, &ops->w, &ops->sb, &ops->bs};
	const int sizes[6] = {q * q, q * q, 2 * q, q, q * q, q * q};
	for (int k = 0; k < 6; ++k) {
		*slots[k] = malloc(sizeof(double) * (size_t)sizes[k]);
		rd(*slots[k], sizeof(double), (size_t)sizes[k], f);
	}

	struct Solver_Volume* vols = calloc((size_t)sim->n_v, sizeof *vols);
	for (int v = 0; v < sim->n_v; ++v) {
		struct Solver_Volume* s = &vols[v];
		s->index = v;
		s->lnk.next = (v + 1 < sim->n_v) ? &vols[v + 1].lnk : NULL;
		ma_init(&s->metrics_vc, 'C', 3, sim->n_vc, d, d);
		ma_init(&s->jacobian_det_vc, 'C', 1, sim->n_vc, 1, 1);
		ma_init(&s->sol_coef, 'C', 2, sim->n_vs, sim->n_var, 1);
		ma_init(&s->rhs, 'C', 2, sim->n_vs, sim->n_var, 1);
		rd(s->metrics_vc.data, sizeof(double), ma_size(&s->metrics_vc), f);
		rd(s->jacobian_det_vc.data, sizeof(double), ma_size(&s->jacobian_det_vc), f);
		rd(s->sol_coef.data, sizeof(double), ma_size(&s->sol_coef), f);
	}
	struct Solver_Face* faces = calloc((size_t)sim->n_f, sizeof *faces);
	for (int i = 0; i < sim->n_f; ++i) {
		struct Solver_Face* s = &faces[i];
		s->index = i;
		s->lnk.next = (i + 1 < sim->n_f) ? &faces[i + 1].lnk : NULL;
		int32_t nb[7];
		rd(nb, sizeof(int32_t), 7, f);
		s->boundary = (nb[1] < 0);
		s->bc = nb[6];
		for (int side = 0; side < 2; ++side) {
			const int v = nb[side];
			if (v < -1 || v >= sim->n_v)
				die("face volume out of range");
			s->neigh_info[side].volume = (v >= 0) ? &vols[v] : NULL;
			s->neigh_info[side].ind_lf = nb[2 + side];
			s->neigh_info[side].ind_ord = nb[4 + side];
		}
		ma_init(&s->normals_fc, 'R', 2, sim->n_fc, d, 1);
		ma_init(&s->jacobian_det_fc, 'C', 1, sim->n_fc, 1, 1);
		rd(s->normals_fc.data, sizeof(double), ma_size(&s->normals_fc), f);
		rd(s->jacobian_det_fc.data, sizeof(double), ma_size(&s->jacobian_det_fc), f);
		if (s->boundary) {
			ma_init(&s->s_bv, 'R', 2, sim->n_fc, sim->n_var, 1);
			rd(s->s_bv.data, sizeof(double), ma_size(&s->s_bv), f);
		}
	}
	double extra;
	if (fread(&extra, sizeof extra, 1, f) == 1)
		die("case file too long");
	fclose(f);
	sim->volumes = sim->n_v ? &vols[0].lnk : NULL;
	sim->faces = sim->n_f ? &faces[0].lnk : NULL;
}

/* ------------------------------------------------------------------------------------------------------------
 * The binding: pack once, then the two replaced entry points.
 * ------------------------------------------------------------------------------------------------------------ */
static dgpu_ctx* g_dgpu = NULL;
static double *g_sol = NULL, *g_rhs = NULL;   /* contiguous sol_coef / rhs blocks in list order */

static void pack_from_sim(const struct Simulation* sim, const struct Operators* o)
{
	const int d = sim->d;
	dgpu_physics phys;
	memset(&phys, 0, sizeof phys);
	phys.d = d;
	phys.pde = sim->pde;
	phys.num_flux = sim->num_flux;
	phys.positivity = sim->positivity;
	for (int k = 0; k < 3; ++k)
		phys.b_adv[k] = sim->b_adv[k];
	phys.viscosity = sim->viscosity;   /* Navier-Stokes: the test case's constants */
	phys.mu = sim->mu;
	phys.Pr = sim->Pr;
	phys.r_s = sim->r_s;
	phys.dTdn = sim->dTdn;

	dgpu_tp_operators ops = {.elem_type = (d == 2 ? DGPU_QUAD : DGPU_HEX), .p = sim->p, .cv0_vs_vc = o->cv0,
	                         .cv1_vs_vc = o->cv1, .cv0_vs_fc = o->cv0_fc, .w_vc = o->w, .ccSB0_vs_vs = o->sb,
	                         .ccBS0_vs_vs = o->bs};

	const size_t vm = (size_t)sim->n_vc * d * d, vj = (size_t)sim->n_vc;
	const size_t fn = (size_t)sim->n_fc * d, fj = (size_t)sim->n_fc;
	double* met = malloc(sizeof(double) * vm * (size_t)sim->n_v);
	double* jac = malloc(sizeof(double) * vj * (size_t)sim->n_v);
	double* nrm = malloc(sizeof(double) * fn * (size_t)sim->n_f);
	double* jf = malloc(sizeof(double) * fj * (size_t)sim->n_f);
	int* fv = malloc(sizeof(int) * 2 * (size_t)sim->n_f);
	int* flf = malloc(sizeof(int) * 2 * (size_t)sim->n_f);
	int* bc = malloc(sizeof(int) * (size_t)sim->n_f);
	const size_t fb = (size_t)sim->n_fc * (size_t)sim->n_var;
	double* sbv = calloc(fb * (size_t)sim->n_f, sizeof(double));
	if (!met || !jac || !nrm || !jf || !fv || !flf || !bc || !sbv)
		die("out of memory");
	int n_bnd = 0;

	int v = 0;
	for (struct Intrusive_Link* c = sim->volumes; c; c = c->next, ++v) {
		const struct Solver_Volume* s = (const struct Solver_Volume*)c;
		if (s->index != v || s->metrics_vc.layout != 'C')
			die("volume list out of order or metrics not column-major");
		memcpy(met + v * vm, s->metrics_vc.data, sizeof(double) * vm);
		memcpy(jac + v * vj, s->jacobian_det_vc.data, sizeof(double) * vj);
	}
	int f = 0;
	for (struct Intrusive_Link* c = sim->faces; c; c = c->next, ++f) {
		const struct Solver_Face* s = (const struct Solver_Face*)c;
		for (int side = 0; side < 2; ++side) {
			const struct Neigh_Info* ni = &s->neigh_info[side];
			fv[2 * f + side] = ni->volume ? ni->volume->index : -1;
			flf[2 * f + side] = ni->volume ? ni->ind_lf : -1;
			/* the right-trace permutation of get_operator__nc_fc_T is the identity for every face of these
			 * aligned meshes; a mesh with other orientations passes its nc_fc rows instead of NULL */
			if (ni->volume && !s->boundary && ni->ind_ord != 0)   /* a boundary face has no orientation (-1) */
				die("this caller packs aligned faces only (ind_ord 0)");
		}
		bc[f] = s->bc;
		if (s->boundary) {   /* constructor_sol_bv's values, for the boundary conditions that read them */
			++n_bnd;
			memcpy(sbv + f * fb, s->s_bv.data, sizeof(double) * fb);
		}
		if (s->normals_fc.layout != 'R')
			die("normals not row-major");
		memcpy(nrm + f * fn, s->normals_fc.data, sizeof(double) * fn);
		memcpy(jf + f * fj, s->jacobian_det_fc.data, sizeof(double) * fj);
	}
	dgpu_mesh mesh;
	memset(&mesh, 0, sizeof mesh);
	mesh.n_volumes = sim->n_v;
	mesh.metrics_vc = met;
	mesh.jacobian_det_vc = jac;
	mesh.n_faces = sim->n_f;
	mesh.face_vol = fv;
	mesh.face_lf = flf;
	mesh.nc_fc = NULL;
	mesh.normals_fc = nrm;
	mesh.jacobian_det_fc = jf;
	if (n_bnd > 0) {
		mesh.bc_fc = bc;
		mesh.bc_state_fc = sbv;
		if (sim->bc_data[0] != 0.0 || sim->bc_data[1] != 0.0)
			mesh.bc_data = sim->bc_data;
	}
	if (dgpu_create(&phys, &ops, &mesh, &g_dgpu) != DGPU_OK) {
		fprintf(stderr, "dgpu_create: %s\n", dgpu_last_error(NULL));
		exit(1);
	}
	/* dgpu_create copied everything: the packed arrays may go */
	free(met); free(jac); free(nrm); free(jf); free(fv); free(flf); free(bc); free(sbv);

	size_t n_state = 0;
	if (dgpu_state_size(g_dgpu, &n_state) != DGPU_OK ||
	    n_state != (size_t)sim->n_v * (size_t)sim->n_vs * (size_t)sim->n_var)
		die("state size");
	g_sol = malloc(sizeof(double) * n_state);
	g_rhs = malloc(sizeof(double) * n_state);
	if (!g_sol || !g_rhs)
		die("out of memory");
}

static void gather(const struct Simulation* sim, double* dst, int rhs)
{
	const size_t n = (size_t)sim->n_vs * (size_t)sim->n_var;
	size_t v = 0;
	for (struct Intrusive_Link* c = sim->volumes; c; c = c->next, ++v) {
		const struct Solver_Volume* s = (const struct Solver_Volume*)c;
		memcpy(dst + v * n, rhs ? s->rhs.data : s->sol_coef.data, sizeof(double) * n);
	}
}

static void scatter(const struct Simulation* sim, const double* src, int rhs)
{
	const size_t n = (size_t)sim->n_vs * (size_t)sim->n_var;
	size_t v = 0;
	for (struct Intrusive_Link* c = sim->volumes; c; c = c->next, ++v) {
		struct Solver_Volume* s = (struct Solver_Volume*)c;
		memcpy(rhs ? s->rhs.data : s->sol_coef.data, src + v * n, sizeof(double) * n);
	}
}

/* src/simulation/solvers/dg/solve_dg.c:130 */
static double compute_rhs_dg(const struct Simulation* sim)
{
	gather(sim, g_sol, 0);
	double max_rhs = 0.0;
	if (dgpu_compute_rhs_host(g_dgpu, g_sol, g_rhs, &max_rhs) != DGPU_OK) {
		fprintf(stderr, "compute_rhs_dg: %s\n", dgpu_last_error(g_dgpu));
		exit(1);
	}
	scatter(sim, g_rhs, 1);
	return max_rhs;
}

/* src/simulation/solvers/solve_explicit.c:252 */
static double time_step_ssp_rk_33(const double dt, const struct Simulation* sim)
{
	gather(sim, g_sol, 0);
	double max_rhs = 0.0;
	const dgpu_status st = dgpu_ssp_rk3_step_host(g_dgpu, dt, g_sol, g_sol, &max_rhs);
	if (st == DGPU_ERR_POSITIVITY) {
		fprintf(stderr, "Average density or pressure approaching 0.0.\n");   /* solve.c:204-208 */
		exit(1);
	} else if (st != DGPU_OK) {
		fprintf(stderr, "time_step_ssp_rk_33: %s\n", dgpu_last_error(g_dgpu));
		exit(1);
	}
	scatter(sim, g_sol, 0);
	return max_rhs;
}

int main(int argc, char** argv)
{
	if (argc != 3) {
		fprintf(stderr, "usage: %s case.bin out.bin\n", argv[0]);
		return 2;
	}
	struct Simulation sim;
	struct Operators ops;
	int n_steps = 0;
	double dt = 0.0;
	memset(&sim, 0, sizeof sim);
	read_case(argv[1], &sim, &ops, &n_steps, &dt);
	pack_from_sim(&sim, &ops);

	FILE* out = fopen(argv[2], "wb");
	if (!out)
		die("cannot open the output file");
	const double max0 = compute_rhs_dg(&sim);
	for (struct Intrusive_Link* c = sim.volumes; c; c = c->next) {
		const struct Solver_Volume* s = (const struct Solver_Volume*)c;
		fwrite(s->rhs.data, sizeof(double), ma_size(&s->rhs), out);
	}
	fwrite(&max0, sizeof max0, 1, out);
	double mx = 0.0;
	for (int t = 0; t < n_steps; ++t)
		mx = time_step_ssp_rk_33(dt, &sim);
	for (struct Intrusive_Link* c = sim.volumes; c; c = c->next) {
		const struct Solver_Volume* s = (const struct Solver_Volume*)c;
		fwrite(s->sol_coef.data, sizeof(double), ma_size(&s->sol_coef), out);
	}
	fwrite(&mx, sizeof mx, 1, out);
	fclose(out);
	if (dgpu_destroy(g_dgpu) != DGPU_OK)
		die("dgpu_destroy");
	printf("dgpu_caller: %d volumes, %d faces, %d steps\n", sim.n_v, sim.n_f, n_steps);
	return 0;
}
