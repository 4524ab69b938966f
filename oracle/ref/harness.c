/* Driver of the reference's own explicit-DG code for parity pins (oracle/_ref only: TEST INFRASTRUCTURE).
 *
 *   dpg_ref_harness <ctrl_name> <out_dir> [--map A L] [--keep-sol] [--adapt-p list.txt] [--state sol.bin]
 *                   [--steps N --dt DT]
 *
 * It sets a simulation up the way the reference's integration tests do (structor_simulation,
 * src/testing/integration/test_integration.c:104-126, then the explicit solver's set-up of
 * solve_explicit, src/simulation/solvers/solve_explicit.c:80-93) and writes, in volume-list and face-list order:
 *   volumes.txt  per volume: index, element type, p_ref, curved, n_vs, n_vc, n_ve
 *   xyz_ve.bin, xyz_vs.bin (solution nodes, constructor_xyz_v), metrics_vc.bin, jacobian_det_vc.bin
 *                (the Solver_Volume's own multiarrays, raw column-major data)
 *   faces.txt    per face: index, boundary, bc, n_fc, then per side: volume index, ind_lf, ind_ord (-1 if none)
 *   normals_fc.bin, jacobian_det_fc.bin, xyz_fc.bin (the Solver_Face's own multiarrays)
 * With --state (the initial sol_coef of every volume, n_vs x n_var column-major, concatenated), it overwrites
 * sol_coef, calls compute_rhs (solve.c:133-149 -> compute_rhs_dg) and writes rhs.bin and max_rhs.txt; with
 * --steps it then runs N steps of time_step_ssp_rk_33 (solve_explicit.c:252-301, compiled from the reference's
 * file below) and writes sol_steps.bin and the per-step max_rhs.
 * --map A L makes the domain's parametric map x,y += A sin(pi x / (L/2)) sin(pi y / (L/2)) (both coordinates),
 * the test case's constructor_xyz for a parametric mesh (geometry_T.c:857-874). Without it a parametric mesh keeps
 * the test case's own map (e.g. constructor_xyz_cylinder_parametric_T of the Taylor-Couette case).
 * --adapt-p reads lines "x y p" and, after the initial solution, adapts the orders the way the reference's
 * integration tests adapt an initial mesh (adapt_initial_mesh_if_required, test_integration.c:253-298: adapt_hp with
 * ADAPT_S_XYZ_VE, src/simulation/solvers/adaptation/adaptation.c:112-133): the volumes with vertex (x, y) move
 * towards order p within the control file's p_ref range (every volume starts at its lower end), and the reference
 * keeps neighbouring orders within one of each other; volumes.txt then lists
 * every volume's order and faces.txt every face's node count at p_f = max of its sides.
 * --keep-sol leaves the test case's constructor_sol in place (only the initial state is replaced): the boundary
 * values that read it (the Riemann faces' exterior state, boundary_euler_T.c) then see the test case's solution. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* time_step_ssp_rk_33 is static in the reference's solve_explicit.c: compile that file here (the recipe leaves its
 * own object out of the link). It brings the headers the rest of this driver needs. */
#include "solve_explicit.c"

#include "computational_elements.h"
#include "geometry.h"
#include "solution.h"
#include "face_solver.h"
#include "element.h"
#include "definitions_mesh.h"
#include "adaptation.h"
#include "definitions_adaptation.h"
#include "multiarray_constructors.h"
#include "vector.h"
#include "vector_constructors.h"

static double g_map_a = 0.0, g_map_l = 10.0;

static const struct const_Multiarray_d* constructor_xyz_sinusoidal
	(const char n_type, const struct const_Multiarray_d* xyz_i, const struct Solver_Volume* s_vol,
	 const struct Simulation* sim)
{
	(void)n_type; (void)s_vol; (void)sim;
	const ptrdiff_t n_n = xyz_i->extents[0];
	struct Multiarray_d* xyz = constructor_empty_Multiarray_d('C',2,(ptrdiff_t[]){n_n,DIM});
	const double* x_i = get_col_const_Multiarray_d(0,xyz_i);
	const double* y_i = get_col_const_Multiarray_d(1,xyz_i);
	double* x = get_col_Multiarray_d(0,xyz);
	double* y = get_col_Multiarray_d(1,xyz);
	const double k = 2.0*M_PI/g_map_l;
	for (ptrdiff_t n = 0; n < n_n; ++n) {
		const double dl = g_map_a*sin(k*x_i[n])*sin(k*y_i[n]);
		x[n] = x_i[n] + dl;
		y[n] = y_i[n] + dl;
	}
	return (const struct const_Multiarray_d*) xyz;
}

/* The test case's set_sol, replaced so that set_initial_solution only sizes sol_coef (n_vs x n_var, zeros): the
 * state is then read from the caller's file. */
static void set_sol_zero(const struct Simulation* sim, struct Solution_Container sol_cont)
{
	const struct const_Multiarray_d* xyz = constructor_xyz_sol(sim,&sol_cont);
	const struct Test_Case* tc = (const struct Test_Case*)sim->test_case_rc->tc;
	struct Multiarray_d* sol = constructor_zero_Multiarray_d('C',2,(ptrdiff_t[]){xyz->extents[0],tc->n_var});
	destructor_const_Multiarray_d(xyz);
	update_Solution_Container_sol(&sol_cont,sol,sim);
	destructor_Multiarray_d(sol);
}

/* The test case's constructor_sol, replaced in the same way (zeros at the given nodes). */
static const struct const_Multiarray_d* constructor_sol_zero(const struct const_Multiarray_d* xyz,
                                                             const struct Simulation* sim)
{
	const struct Test_Case* tc = (const struct Test_Case*)sim->test_case_rc->tc;
	return (const struct const_Multiarray_d*)
		constructor_zero_Multiarray_d('C',2,(ptrdiff_t[]){xyz->extents[0],tc->n_var});
}

static FILE* open_out(const char* dir, const char* name, const char* mode)
{
	char path[4096];
	snprintf(path,sizeof(path),"%s/%s",dir,name);
	FILE* f = fopen(path,mode);
	if (!f) {
		fprintf(stderr,"cannot open %s\n",path);
		exit(2);
	}
	return f;
}

static ptrdiff_t ma_size(const struct const_Multiarray_d* a)
{
	return compute_size(a->order,a->extents);
}

static void write_ma(FILE* f, const struct const_Multiarray_d* a)
{
	fwrite(a->data,sizeof(double),(size_t)ma_size(a),f);
}

static void dump_geometry(const struct Simulation* sim, const char* out)
{
	FILE* fv = open_out(out,"volumes.txt","w");
	FILE* fxve = open_out(out,"xyz_ve.bin","wb");
	FILE* fxvs = open_out(out,"xyz_vs.bin","wb");
	FILE* fm = open_out(out,"metrics_vc.bin","wb");
	FILE* fj = open_out(out,"jacobian_det_vc.bin","wb");
	for (struct Intrusive_Link* curr = sim->volumes->first; curr; curr = curr->next) {
		struct Volume* vol = (struct Volume*) curr;
		struct Solver_Volume* s_vol = (struct Solver_Volume*) curr;
		const struct const_Multiarray_d* xyz_vs = constructor_xyz_v(sim,s_vol,'s',false);
		fprintf(fv,"%d %d %d %d %td %td %td\n",vol->index,vol->element->type,s_vol->p_ref,(int)vol->curved,
		        xyz_vs->extents[0],s_vol->jacobian_det_vc->extents[0],vol->xyz_ve->extents[0]);
		write_ma(fxve,vol->xyz_ve);
		write_ma(fxvs,xyz_vs);
		write_ma(fm,s_vol->metrics_vc);
		write_ma(fj,s_vol->jacobian_det_vc);
		destructor_const_Multiarray_d(xyz_vs);
	}
	fclose(fv); fclose(fxve); fclose(fxvs); fclose(fm); fclose(fj);

	FILE* ff = open_out(out,"faces.txt","w");
	FILE* fn = open_out(out,"normals_fc.bin","wb");
	FILE* fjf = open_out(out,"jacobian_det_fc.bin","wb");
	FILE* fxf = open_out(out,"xyz_fc.bin","wb");
	for (struct Intrusive_Link* curr = sim->faces->first; curr; curr = curr->next) {
		struct Face* face = (struct Face*) curr;
		struct Solver_Face* s_face = (struct Solver_Face*) curr;
		fprintf(ff,"%d %d %d %td",face->index,(int)face->boundary,face->bc,s_face->jacobian_det_fc->extents[0]);
		for (int s = 0; s < 2; ++s) {
			const struct Neigh_Info* ni = &face->neigh_info[s];
			if (ni->volume)
				fprintf(ff," %d %d %d",ni->volume->index,ni->ind_lf,ni->ind_ord);
			else
				fprintf(ff," -1 -1 -1");
		}
		fprintf(ff,"\n");
		write_ma(fn,s_face->normals_fc);
		write_ma(fjf,s_face->jacobian_det_fc);
		write_ma(fxf,s_face->xyz_fc);
	}
	fclose(ff); fclose(fn); fclose(fjf); fclose(fxf);
}

static void adapt_orders(struct Simulation* sim, const char* path)
{
	FILE* f = fopen(path,"r");
	if (!f) {
		fprintf(stderr,"cannot open %s\n",path);
		exit(2);
	}
	int n = 0;
	double x, y;
	int p;
	while (fscanf(f,"%lf %lf %d",&x,&y,&p) == 3)
		++n;
	rewind(f);
	struct Multiarray_d* xyz = constructor_empty_Multiarray_d('R',2,(ptrdiff_t[]){n,2});
	struct Vector_i* ps = constructor_empty_Vector_i(n);
	for (int i = 0; i < n; ++i) {
		if (fscanf(f,"%lf %lf %d",&x,&y,&p) != 3)
			exit(2);
		xyz->data[2*i] = x;
		xyz->data[2*i+1] = y;
		ps->data[i] = p;
	}
	fclose(f);
	struct Adaptation_Data adapt_data = { .adapt_h = { 0, 0, }, .xyz_ve_refine = (const struct const_Multiarray_d*)xyz,
	                                      .xyz_ve_ml = NULL, .xyz_ve_p = (const struct const_Vector_i*)ps, };
	adapt_hp(sim,ADAPT_S_XYZ_VE,&adapt_data);
	destructor_Multiarray_d(xyz);
	destructor_Vector_i(ps);
}

static void read_state(const struct Simulation* sim, const char* path)
{
	FILE* f = fopen(path,"rb");
	if (!f) {
		fprintf(stderr,"cannot open %s\n",path);
		exit(2);
	}
	for (struct Intrusive_Link* curr = sim->volumes->first; curr; curr = curr->next) {
		struct Multiarray_d* s = ((struct Solver_Volume*) curr)->sol_coef;
		const size_t n = (size_t)compute_size(s->order,s->extents);
		if (fread(s->data,sizeof(double),n,f) != n) {
			fprintf(stderr,"state file too short\n");
			exit(2);
		}
	}
	double extra;
	if (fread(&extra,sizeof(double),1,f) == 1) {
		fprintf(stderr,"state file too long\n");
		exit(2);
	}
	fclose(f);
}

static void write_volume_field(const struct Simulation* sim, FILE* f, int which)
{
	for (struct Intrusive_Link* curr = sim->volumes->first; curr; curr = curr->next) {
		struct Solver_Volume* s_vol = (struct Solver_Volume*) curr;
		write_ma(f,(const struct const_Multiarray_d*)(which == 0 ? s_vol->rhs : s_vol->sol_coef));
	}
}

int main(int argc, char** argv)
{
	if (argc < 3) {
		fprintf(stderr,"usage: %s ctrl_name out_dir [--map A L] [--keep-sol] [--adapt-p list.txt] [--state sol.bin] "
		        "[--steps N --dt DT]\n",
		        argv[0]);
		return 2;
	}
	const char* ctrl_name = argv[1];
	const char* out = argv[2];
	const char* state = NULL;
	int n_steps = 0;
	double dt = 0.0;
	int keep_sol = 0;
	const char* adapt_p = NULL;
	for (int i = 3; i < argc; ++i) {
		if (!strcmp(argv[i],"--keep-sol")) {
			keep_sol = 1;
		} else if (!strcmp(argv[i],"--adapt-p") && i + 1 < argc) {
			adapt_p = argv[++i];
		} else if (!strcmp(argv[i],"--map") && i + 2 < argc) {
			g_map_a = atof(argv[++i]);
			g_map_l = atof(argv[++i]);
		} else if (!strcmp(argv[i],"--state") && i + 1 < argc) {
			state = argv[++i];
		} else if (!strcmp(argv[i],"--steps") && i + 1 < argc) {
			n_steps = atoi(argv[++i]);
		} else if (!strcmp(argv[i],"--dt") && i + 1 < argc) {
			dt = atof(argv[++i]);
		} else {
			fprintf(stderr,"unknown argument %s\n",argv[i]);
			return 2;
		}
	}

	/* structor_simulation(..., 'c', ADAPT_0, ..., 'r', ...) of test_integration.c:104-126. */
	struct Simulation* sim = constructor_Simulation(ctrl_name);
	struct Test_Case* test_case = (struct Test_Case*)sim->test_case_rc->tc;
	if (sim->domain_type == DOM_PARAMETRIC && g_map_a != 0.0)
		test_case->constructor_xyz = constructor_xyz_sinusoidal;
	test_case->set_sol = test_case->set_sol_start = set_sol_zero;
	if (!keep_sol)
		test_case->constructor_sol = test_case->constructor_sol_start = constructor_sol_zero;
	constructor_derived_Elements(sim,IL_ELEMENT_SOLVER);
	constructor_derived_computational_elements(sim,IL_SOLVER);
	set_up_solver_geometry(sim);
	set_initial_solution(sim);
	if (adapt_p)
		adapt_orders(sim,adapt_p);

	dump_geometry(sim,out);

	if (state) {
		/* solve_explicit's set-up (solve_explicit.c:80-93) with the given initial state. */
		test_case->solver_method_curr = 'e';
		test_case->time = 0.0;
		constructor_derived_Elements(sim,IL_ELEMENT_SOLVER_DG);
		constructor_derived_computational_elements(sim,IL_SOLVER_DG);
		read_state(sim,state);

		const double max_rhs = compute_rhs(sim);
		FILE* fr = open_out(out,"rhs.bin","wb");
		write_volume_field(sim,fr,0);
		fclose(fr);
		FILE* fmx = open_out(out,"max_rhs.txt","w");
		fprintf(fmx,"%.17g\n",max_rhs);

		if (n_steps > 0) {
			read_state(sim,state);
			for (int t = 0; t < n_steps; ++t) {
				test_case->time += dt;
				fprintf(fmx,"%.17g\n",time_step_ssp_rk_33(dt,sim));
			}
			FILE* fs = open_out(out,"sol_steps.bin","wb");
			write_volume_field(sim,fs,1);
			fclose(fs);
		}
		fclose(fmx);
	}
	return 0;
}
