/* A C11 host program that calls the batched (mixed-order) residual through include/dgpu.h the way DPGSolver's C code
 * would after its p-adaptation (adapt_hp, src/simulation/solvers/adaptation/adaptation.c:112-133): every solver
 * volume carries its own order p_ref and every face its node count at p_f = max(p_L, p_R) (face_solver.c:123-132).
 * The program holds the lists with the reference's multiarrays, packs them once in list order (ragged blocks), keeps
 * one TP operator set per order (the reference indexes its element operators by p, element_solver.h:31-74), and
 * replaces compute_rhs_dg (solve_dg.c:130-136) and time_step_ssp_rk_33 (solve_explicit.c:252-301).
 *
 *     dgpu_batch_caller <case.bin> <out.bin>
 *
 * case.bin (little endian, written by tests/test_gpu_c_caller.py):
 *   int32  magic 0x48435442, d, pde, num_flux, positivity, n_groups, n_volumes, n_faces, n_steps
 *   f64    dt, b_adv[3]
 *   int32  viscosity; f64 mu, Pr, r_s, dTdn; f64 bc_data[4]; int32 has_source
 *   per group: int32 p; f64 cv0_vs_vc (q x q), cv1_vs_vc (q x q), cv0_vs_fc (2 x q), w_vc (q), ccSB0, ccBS0 (q x q)
 *   per volume: int32 group; f64 metrics_vc (n_vc, d, d) 'C', jacobian_det_vc (n_vc), sol_coef (n_vs, n_var) 'C';
 *               with has_source also the test case's source at its cubature nodes (n_vc, n_var) 'C'
 *   per face:   int32 volume[2], ind_lf[2], bc, n_fc; f64 normals_fc (n_fc, d) 'R', jacobian_det_fc (n_fc); on a
 *               boundary face also the exterior state (n_fc, n_var) 'R'
 * out.bin: per volume rhs (n_vs, n_var) 'C' after compute_rhs_dg, then f64 max_rhs; per volume sol_coef after
 * n_steps calls of time_step_ssp_rk_33 (one batched call), then f64 max_rhs of the last step.
 */
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dgpu.h"

struct Multiarray_d {
	char layout;
	int order;
	ptrdiff_t extents[3];
	double* data;
};

struct Intrusive_Link {
	struct Intrusive_Link* next;
};

struct Solver_Volume {
	struct Intrusive_Link lnk;
	int index, p_ref, group;
	struct Multiarray_d sol_coef, rhs, metrics_vc, jacobian_det_vc;
	struct Multiarray_d source;   /* the test case's source at the cubature nodes (compute_source_rhs_dg_like) */
};

struct Solver_Face {
	struct Intrusive_Link lnk;
	int index, boundary, bc, n_fc;
	int vol[2], ind_lf[2];
	struct Multiarray_d normals_fc, jacobian_det_fc, s_bv;
};

struct Group {
	int p;
	double *cv0, *cv1, *cv0_fc, *w, *sb, *bs;
};

struct Simulation {
	int d, pde, num_flux, positivity, n_var, n_g, n_v, n_f, has_source;
	double b_adv[3];
	int viscosity;
	double mu, Pr, r_s, dTdn, bc_data[4];
	struct Group* groups;
	struct Intrusive_Link* volumes;
	struct Intrusive_Link* faces;
};

static void die(const char* what)
{
	fprintf(stderr, "dgpu_batch_caller: %s\n", what);
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

static int n_nodes(int d, int p) { return d == 2 ? (p + 1) * (p + 1) : (p + 1) * (p + 1) * (p + 1); }

static void read_case(const char* path, struct Simulation* sim, int* n_steps, double* dt)
{
	FILE* f = fopen(path, "rb");
	if (!f)
		die("cannot open the case file");
	int32_t h[9];
	rd(h, sizeof(int32_t), 9, f);
	if (h[0] != 0x48435442)
		die("bad magic");
	sim->d = h[1];
	sim->pde = h[2];
	sim->num_flux = h[3];
	sim->positivity = h[4];
	sim->n_g = h[5];
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
	int32_t has_source;
	rd(&has_source, sizeof has_source, 1, f);
	sim->has_source = has_source != 0;
	sim->viscosity = visc;
	sim->mu = nsc[0];
	sim->Pr = nsc[1];
	sim->r_s = nsc[2];
	sim->dTdn = nsc[3];
	const int d = sim->d;
	sim->n_var = (sim->pde == DGPU_PDE_ADVECTION ? 1 : d + 2);

	sim->groups = calloc((size_t)sim->n_g, sizeof *sim->groups);
	for (int g = 0; g < sim->n_g; ++g) {
		struct Group* G = &sim->groups[g];
		int32_t p;
		rd(&p, sizeof p, 1, f);
		if (p < 1 || p > 4)
			die("order out of range");
		G->p = p;
		const int q = p + 1;
		double** slots[6] = {&G->cv0, &G->cv1, &G->cv0_fc, &G->w, &G->sb, &G->bs};
		const int sizes[6] = {q * q, q * q, 2 * q, q, q * q, q * q};
		for (int k = 0; k < 6; ++k) {
			*slots[k] = malloc(sizeof(double) * (size_t)sizes[k]);
			rd(*slots[k], sizeof(double), (size_t)sizes[k], f);
		}
	}
	struct Solver_Volume* vols = calloc((size_t)sim->n_v, sizeof *vols);
	for (int v = 0; v < sim->n_v; ++v) {
		struct Solver_Volume* s = &vols[v];
		int32_t g;
		rd(&g, sizeof g, 1, f);
		if (g < 0 || g >= sim->n_g)
			die("group out of range");
		s->index = v;
		s->group = g;
		s->p_ref = sim->groups[g].p;
		s->lnk.next = (v + 1 < sim->n_v) ? &vols[v + 1].lnk : NULL;
		const int n = n_nodes(d, s->p_ref);
		ma_init(&s->metrics_vc, 'C', 3, n, d, d);
		ma_init(&s->jacobian_det_vc, 'C', 1, n, 1, 1);
		ma_init(&s->sol_coef, 'C', 2, n, sim->n_var, 1);
		ma_init(&s->rhs, 'C', 2, n, sim->n_var, 1);
		rd(s->metrics_vc.data, sizeof(double), ma_size(&s->metrics_vc), f);
		rd(s->jacobian_det_vc.data, sizeof(double), ma_size(&s->jacobian_det_vc), f);
		rd(s->sol_coef.data, sizeof(double), ma_size(&s->sol_coef), f);
		if (sim->has_source) {
			ma_init(&s->source, 'C', 2, n, sim->n_var, 1);
			rd(s->source.data, sizeof(double), ma_size(&s->source), f);
		}
	}
	struct Solver_Face* faces = calloc((size_t)sim->n_f, sizeof *faces);
	for (int i = 0; i < sim->n_f; ++i) {
		struct Solver_Face* s = &faces[i];
		int32_t nb[6];
		rd(nb, sizeof(int32_t), 6, f);
		s->index = i;
		s->lnk.next = (i + 1 < sim->n_f) ? &faces[i + 1].lnk : NULL;
		for (int side = 0; side < 2; ++side) {
			if (nb[side] < -1 || nb[side] >= sim->n_v)
				die("face volume out of range");
			s->vol[side] = nb[side];
			s->ind_lf[side] = nb[2 + side];
		}
		s->boundary = nb[1] < 0;
		s->bc = nb[4];
		s->n_fc = nb[5];
		ma_init(&s->normals_fc, 'R', 2, s->n_fc, d, 1);
		ma_init(&s->jacobian_det_fc, 'C', 1, s->n_fc, 1, 1);
		rd(s->normals_fc.data, sizeof(double), ma_size(&s->normals_fc), f);
		rd(s->jacobian_det_fc.data, sizeof(double), ma_size(&s->jacobian_det_fc), f);
		if (s->boundary) {
			ma_init(&s->s_bv, 'R', 2, s->n_fc, sim->n_var, 1);
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
 * pack_from_sim for a p-adapted mesh: ragged per-volume and per-face blocks concatenated in list order.
 * ------------------------------------------------------------------------------------------------------------ */
static dgpu_batch* g_batch;
static size_t g_n_state;

static double* cat_volumes(const struct Simulation* sim, size_t offset_of_ma)
{
	size_t n = 0;
	for (struct Intrusive_Link* c = sim->volumes; c; c = c->next)
		n += ma_size((const struct Multiarray_d*)((const char*)c + offset_of_ma));
	double* out = malloc(sizeof(double) * (n ? n : 1));
	size_t o = 0;
	for (struct Intrusive_Link* c = sim->volumes; c; c = c->next) {
		const struct Multiarray_d* a = (const struct Multiarray_d*)((const char*)c + offset_of_ma);
		memcpy(out + o, a->data, sizeof(double) * ma_size(a));
		o += ma_size(a);
	}
	return out;
}

static double* cat_faces(const struct Simulation* sim, size_t offset_of_ma, int boundary_only)
{
	size_t n = 0;
	for (struct Intrusive_Link* c = sim->faces; c; c = c->next) {
		const struct Solver_Face* s = (const struct Solver_Face*)c;
		const struct Multiarray_d* a = (const struct Multiarray_d*)((const char*)c + offset_of_ma);
		n += (boundary_only && !s->boundary) ? (size_t)s->n_fc * (size_t)sim->n_var : ma_size(a);
	}
	double* out = calloc(n ? n : 1, sizeof(double));
	size_t o = 0;
	for (struct Intrusive_Link* c = sim->faces; c; c = c->next) {
		const struct Solver_Face* s = (const struct Solver_Face*)c;
		const struct Multiarray_d* a = (const struct Multiarray_d*)((const char*)c + offset_of_ma);
		if (boundary_only && !s->boundary) {   /* interior faces: zeros, never read */
			o += (size_t)s->n_fc * (size_t)sim->n_var;
			continue;
		}
		memcpy(out + o, a->data, sizeof(double) * ma_size(a));
		o += ma_size(a);
	}
	return out;
}

static void pack_from_sim(const struct Simulation* sim)
{
	dgpu_physics phys;
	memset(&phys, 0, sizeof phys);
	phys.d = sim->d;
	phys.pde = sim->pde;
	phys.num_flux = sim->num_flux;
	phys.positivity = sim->positivity;
	memcpy(phys.b_adv, sim->b_adv, sizeof phys.b_adv);
	phys.viscosity = sim->viscosity;
	phys.mu = sim->mu;
	phys.Pr = sim->Pr;
	phys.r_s = sim->r_s;
	phys.dTdn = sim->dTdn;

	dgpu_tp_operators* ops = calloc((size_t)sim->n_g, sizeof *ops);
	for (int g = 0; g < sim->n_g; ++g) {
		const struct Group* G = &sim->groups[g];
		ops[g].elem_type = sim->d == 2 ? DGPU_QUAD : DGPU_HEX;
		ops[g].p = G->p;
		ops[g].cv0_vs_vc = G->cv0;
		ops[g].cv1_vs_vc = G->cv1;
		ops[g].cv0_vs_fc = G->cv0_fc;
		ops[g].w_vc = G->w;
		ops[g].ccSB0_vs_vs = G->sb;
		ops[g].ccBS0_vs_vs = G->bs;
	}
	int* vol_group = malloc(sizeof(int) * (size_t)sim->n_v);
	for (struct Intrusive_Link* c = sim->volumes; c; c = c->next) {
		const struct Solver_Volume* s = (const struct Solver_Volume*)c;
		vol_group[s->index] = s->group;
	}
	int* face_vol = malloc(sizeof(int) * 2 * (size_t)sim->n_f);
	int* face_lf = malloc(sizeof(int) * 2 * (size_t)sim->n_f);
	int* bc_fc = malloc(sizeof(int) * (size_t)sim->n_f);
	int any_boundary = 0;
	for (struct Intrusive_Link* c = sim->faces; c; c = c->next) {
		const struct Solver_Face* s = (const struct Solver_Face*)c;
		for (int side = 0; side < 2; ++side) {
			face_vol[2 * s->index + side] = s->vol[side];
			face_lf[2 * s->index + side] = s->boundary && side == 1 ? -1 : s->ind_lf[side];
		}
		bc_fc[s->index] = s->boundary ? s->bc : 0;
		any_boundary |= s->boundary;
	}
	dgpu_mesh mesh;
	memset(&mesh, 0, sizeof mesh);
	mesh.n_volumes = sim->n_v;
	mesh.metrics_vc = cat_volumes(sim, offsetof(struct Solver_Volume, metrics_vc));
	mesh.jacobian_det_vc = cat_volumes(sim, offsetof(struct Solver_Volume, jacobian_det_vc));
	mesh.n_faces = sim->n_f;
	mesh.face_vol = face_vol;
	mesh.face_lf = face_lf;
	mesh.nc_fc = NULL;   /* straight, aligned QUAD frames: every right-trace permutation is the identity */
	mesh.normals_fc = cat_faces(sim, offsetof(struct Solver_Face, normals_fc), 0);
	mesh.jacobian_det_fc = cat_faces(sim, offsetof(struct Solver_Face, jacobian_det_fc), 0);
	if (any_boundary) {
		mesh.bc_fc = bc_fc;
		mesh.bc_state_fc = cat_faces(sim, offsetof(struct Solver_Face, s_bv), 1);
		mesh.bc_data = sim->bc_data;
	}
	if (dgpu_batch_create(&phys, sim->n_g, ops, vol_group, &mesh, &g_batch) != DGPU_OK)
		die(dgpu_batch_last_error(g_batch));
	if (dgpu_batch_state_size(g_batch, &g_n_state) != DGPU_OK)
		die("dgpu_batch_state_size");
	if (sim->has_source) {   /* compute_source_rhs_dg_like, solve_dg.c:188 */
		double* src = cat_volumes(sim, offsetof(struct Solver_Volume, source));
		if (dgpu_batch_set_source(g_batch, src) != DGPU_OK)
			die(dgpu_batch_last_error(g_batch));
		free(src);
	}
	/* the context keeps its own copies */
	free(ops);
	free(vol_group);
	free(face_vol);
	free(face_lf);
	free(bc_fc);
	free((void*)mesh.metrics_vc);
	free((void*)mesh.jacobian_det_vc);
	free((void*)mesh.normals_fc);
	free((void*)mesh.jacobian_det_fc);
	free((void*)mesh.bc_state_fc);
}

/* ------------------------------------------------------------------------------------------------------------
 * The two entry points, on the volumes' sol_coef / rhs.
 * ------------------------------------------------------------------------------------------------------------ */
static void scatter(const struct Simulation* sim, const double* flat, size_t offset_of_ma)
{
	size_t o = 0;
	for (struct Intrusive_Link* c = sim->volumes; c; c = c->next) {
		struct Multiarray_d* a = (struct Multiarray_d*)((char*)c + offset_of_ma);
		memcpy(a->data, flat + o, sizeof(double) * ma_size(a));
		o += ma_size(a);
	}
}

static double compute_rhs_dg(const struct Simulation* sim)
{
	double* u = cat_volumes(sim, offsetof(struct Solver_Volume, sol_coef));
	double* r = malloc(sizeof(double) * g_n_state);
	double mx = 0.0;
	if (dgpu_batch_upload_state(g_batch, u) != DGPU_OK || dgpu_batch_compute_rhs(g_batch, &mx) != DGPU_OK ||
	    dgpu_batch_download_rhs(g_batch, r) != DGPU_OK)
		die(dgpu_batch_last_error(g_batch));
	scatter(sim, r, offsetof(struct Solver_Volume, rhs));
	free(u);
	free(r);
	return mx;
}

static double time_step_ssp_rk_33_n(const struct Simulation* sim, double dt, int n_steps)
{
	double* u = cat_volumes(sim, offsetof(struct Solver_Volume, sol_coef));
	double mx = 0.0;
	if (dgpu_batch_upload_state(g_batch, u) != DGPU_OK || dgpu_batch_ssp_rk3_steps(g_batch, dt, n_steps, &mx) != DGPU_OK ||
	    dgpu_batch_download_state(g_batch, u) != DGPU_OK)
		die(dgpu_batch_last_error(g_batch));
	scatter(sim, u, offsetof(struct Solver_Volume, sol_coef));
	free(u);
	return mx;
}

int main(int argc, char** argv)
{
	if (argc != 3) {
		fprintf(stderr, "usage: %s case.bin out.bin\n", argv[0]);
		return 2;
	}
	struct Simulation sim;
	int n_steps = 0;
	double dt = 0.0;
	memset(&sim, 0, sizeof sim);
	read_case(argv[1], &sim, &n_steps, &dt);
	pack_from_sim(&sim);

	FILE* out = fopen(argv[2], "wb");
	if (!out)
		die("cannot open the output file");
	const double max0 = compute_rhs_dg(&sim);
	for (struct Intrusive_Link* c = sim.volumes; c; c = c->next) {
		const struct Solver_Volume* s = (const struct Solver_Volume*)c;
		fwrite(s->rhs.data, sizeof(double), ma_size(&s->rhs), out);
	}
	fwrite(&max0, sizeof max0, 1, out);
	const double mx = time_step_ssp_rk_33_n(&sim, dt, n_steps);
	for (struct Intrusive_Link* c = sim.volumes; c; c = c->next) {
		const struct Solver_Volume* s = (const struct Solver_Volume*)c;
		fwrite(s->sol_coef.data, sizeof(double), ma_size(&s->sol_coef), out);
	}
	fwrite(&mx, sizeof mx, 1, out);
	fclose(out);
	if (dgpu_batch_destroy(g_batch) != DGPU_OK)
		die("dgpu_batch_destroy");
	printf("dgpu_batch_caller: %d volumes in %d orders, %d faces, %d steps\n", sim.n_v, sim.n_g, sim.n_f, n_steps);
	return 0;
}
