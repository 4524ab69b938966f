// C ABI of the GB300 explicit DG residual (declared in include/dgpu.h).
//
// Host side: validates and packs the caller's operators and geometry once (dgpu_create), owns all device
// memory, launches the TP kernels of dgpu_tp.cuh on one stream per context, and replays each SSP-RK3 step
// from a captured CUDA graph.
#include <cuda_runtime.h>

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/dgpu.h"
#include "dgpu_tp.cuh"
#include "dgpu_adjoint.cuh"
#include "dgpu_geometry.cuh"
#include "dgpu_jacobian.cuh"
#include "dgpu_ns.cuh"
#include "dgpu_ns_adjoint.cuh"
#include "dgpu_jvp.cuh"
#include "dgpu_host_ops.h"

using namespace dgpu;

namespace {

thread_local std::string g_create_error;


struct KernelTimer {
	const char* name;
	cudaEvent_t start, stop;
};

}  // namespace

struct dgpu_ctx {
	// problem
	int d = 0, q = 0, N = 0, NF = 0, nv = 0, pde = 0, flux = 0, positivity = 0;
	int n_vol = 0, n_face = 0;
	double b_adv[3] = {0, 0, 0};
	TPOps ops;
	// device memory
	double *u = nullptr, *u0 = nullptr, *rhs = nullptr;
	double* ug = nullptr;                 // state as GL nodal values (time stepping); u0 holds the stage-0 copy
	// adjoint (allocated on first use): state kept by dgpu_vjp_forward, cotangent, gradient, adjoint face data
	double *u_saved = nullptr, *vbar = nullptr, *ubar = nullptr, *atraces = nullptr, *wbar = nullptr;
	int* obj_faces = nullptr;             // faces of the objective J (side 0), see dgpu_set_objective_faces
	int n_obj = 0;
	double* obj_contrib = nullptr;        // per objective face node: w_f J_f p
	// forward-mode linearisation (allocated on first use): tangent state, volume term, traces, face fluxes, product
	double *jv_du = nullptr, *jv_vol = nullptr, *jv_traces = nullptr, *jv_nnf = nullptr, *jv_out = nullptr;
	// block-sparse Jacobian (built on first use): block rows, colouring, block slot of (volume, colour)
	std::vector<int> h_face_vol;          // host copy of face_vol
	// element partition (face sides of other ranks' volumes, DGPU_REMOTE_VOLUME): the halo plan of dgpu_halo_setup
	int n_remote = 0;                     // face sides whose volume belongs to another rank
	int n_halo = 0;                       // trace slots exchanged per stage
	int *halo_send = nullptr, *halo_recv = nullptr;   // slots 2f+s: the local side of a cut face / its remote side
	double *halo_sbuf = nullptr, *halo_rbuf = nullptr;   // n_halo x (nv x NF): what is sent / what arrives
	bool halo_recv_ready = false;
	int jac_colours = 0;
	std::vector<int> jac_row_ptr, jac_col_idx, jac_members_off;
	int *jac_slot = nullptr, *jac_members = nullptr;
	bool coef_valid = true, gl_valid = false;   // which of u / ug holds the current state
	double *gmet = nullptr, *inv_wJ = nullptr, *fgeo = nullptr;
	int *vol_face = nullptr, *nc = nullptr, *nc_inv = nullptr;
	bool ns = false;                      // Navier-Stokes: BR2 gradient buffers and the four-kernel stage
	NsPhys ns_phys = {0.0, 1.0, 1.0, 101, 0.0};
	double *ns_gtr = nullptr, *ns_lam = nullptr, *ns_X = nullptr, *ns_gv = nullptr;
	double *ns_gtr_d = nullptr, *ns_X_d = nullptr, *ns_gv_d = nullptr;   // their tangents (linearisations)
	double *ns_gbar = nullptr, *ns_xbar = nullptr, *ns_gtbar = nullptr;  // cotangents (VJP, dgpu_ns_adjoint.cuh)
	int stage_launches = 3;               // kernels per residual evaluation / RK stage
	int n_bnd = 0;                        // boundary faces (face_vol[2f+1] < 0)
	int *bnd = nullptr, *bc_code = nullptr;
	double* bc_ext = nullptr;
	BcData bc_data = {0.0, 0.0, 0.0, 0.0};
	double *traces = nullptr, *nnf = nullptr, *vol_gl = nullptr;
	unsigned long long* max_bits = nullptr;
	int* err_flag = nullptr;
	unsigned long long* n_corr = nullptr;
	double* source = nullptr;             // the test case's source at the cubature nodes (dgpu_set_source), or null
	// execution
	cudaStream_t stream = nullptr;
	bool own_stream = false;
	cudaGraphExec_t rk_graph = nullptr;       // one SSP-RK3 step
	cudaGraphExec_t rk_graph_max = nullptr;   // the same step reducing max|rhs| in its last stage
	double rk_graph_dt = 0.0, rk_graph_max_dt = 0.0;
	// dgpu_ssp_rk3_step_host: a step that reads and writes caller buffers, captured for one (dt, in, out, max)
	cudaGraphExec_t host_graph = nullptr;
	double host_graph_dt = 0.0;
	const double* host_graph_in = nullptr;
	double* host_graph_out = nullptr;
	bool host_graph_max = false;
	long long launches = 0;
	std::string err;
	// launchers for the instantiated (D, Q, NV, PDE, FLUX)
	cudaError_t (*launch_volume)(dgpu_ctx*) = nullptr;      // input: GLL coefficients u
	cudaError_t (*launch_volume_gl)(dgpu_ctx*) = nullptr;   // input: GL nodal values ug
	cudaError_t (*launch_face)(dgpu_ctx*) = nullptr;
	cudaError_t (*launch_lift_rhs)(dgpu_ctx*) = nullptr;
	cudaError_t (*launch_lift_rk)(dgpu_ctx*, double dt, int stage, int want_max) = nullptr;
	// the first volume term of a step on GLL coefficients `in`, keeping them (keep_coef, may be null) and ug; the
	// last lift also writing the new coefficients to u and out_host (may be null). Null for Navier-Stokes.
	cudaError_t (*launch_volume_in)(dgpu_ctx*, const double* in, double* keep_coef) = nullptr;
	cudaError_t (*launch_lift_out)(dgpu_ctx*, double dt, int want_max, double* out_host) = nullptr;
	// basis change of a whole state between GLL coefficients and GL values; in_copy / out_copy may be null
	cudaError_t (*launch_convert)(dgpu_ctx*, bool to_gl, const double* in, double* out, double* in_copy,
	                              double* out_copy) = nullptr;
	cudaError_t (*launch_adjoint)(dgpu_ctx*, const double* u, const double* rbar, double* ubar) = nullptr;
	cudaError_t (*launch_objective)(dgpu_ctx*, double* ubar) = nullptr;   // needs traces of the state
	cudaError_t (*launch_jvp)(dgpu_ctx*) = nullptr;   // R(u) into rhs and (dR/du) jv_du into jv_out
	cudaError_t (*launch_jvp_tangent)(dgpu_ctx*) = nullptr;   // (dR/du) jv_du into jv_out only
	cudaError_t (*launch_mass)(dgpu_ctx*, const double* in, double* out) = nullptr;   // out = M in per volume
	// optional per-kernel timing (eager launches only)
	bool timing = false;
	std::vector<KernelTimer> timers;

	TPParams params() const
	{
		TPParams P;
		P.n_vol = n_vol;
		P.n_face = n_face;
		P.b_adv[0] = b_adv[0];
		P.b_adv[1] = b_adv[1];
		P.b_adv[2] = b_adv[2];
		P.vol_face = vol_face;
		P.gmet = gmet;
		P.inv_wJ = inv_wJ;
		P.fgeo = fgeo;
		P.nc = nc;
		P.nc_inv = nc_inv;
		P.traces = traces;
		P.nnf = nnf;
		P.vol_gl = vol_gl;
		P.max_bits = max_bits;
		P.err_flag = err_flag;
		P.n_corr = n_corr;
		P.bnd = bnd;
		P.bc_code = bc_code;
		P.bc_ext = bc_ext;
		P.bc_data = bc_data;
		P.ns_gtr = ns_gtr;
		P.ns_lam = ns_lam;
		P.ns_X = ns_X;
		P.ns_gv = ns_gv;
		P.ns = ns_phys;
		P.ns_eta = 1.01 * 2 * d;   // PENALTY_SCALING * NFMAX (compute_face_rlhs_dg_T.c:273-295)
		P.source = source;
		return P;
	}
};

namespace {

dgpu_status fail(dgpu_ctx* c, dgpu_status st, const std::string& msg)
{
	if (c)
		c->err = msg;
	else
		g_create_error = msg;
	return st;
}

dgpu_status cuda_fail(dgpu_ctx* c, cudaError_t e, const char* what)
{
	std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
	return fail(c, DGPU_ERR_CUDA, m);
}

#define DGPU_CUDA(ctx, call)                                   \
	do {                                                       \
		cudaError_t e_ = (call);                               \
		if (e_ != cudaSuccess)                                 \
			return cuda_fail((ctx), e_, #call);                \
	} while (0)


template <int D, int Q, int NV>
size_t volume_smem_bytes()
{
	using S = TPShape<D, Q>;
	return (sizeof(TPOps) + 7) / 8 * 8 + (size_t)S::E * (NV * S::N * 2 + D * NV * S::N) * sizeof(double);
}

template <int D, int Q, int NV>
size_t lift_smem_bytes()
{
	using S = TPShape<D, Q>;
	return (sizeof(TPOps) + 7) / 8 * 8 + (size_t)S::E * (3 * NV * S::N + 8) * sizeof(double);
}

template <int D, int Q, int NV>
size_t adj_volume_smem_bytes()
{
	using S = TPShape<D, Q>;
	return (sizeof(TPOps) + 7) / 8 * 8 + (size_t)S::E * (3 * NV * S::N + D * NV * S::N) * sizeof(double);
}

template <int D, int Q, int NV>
size_t convert_smem_bytes()
{
	using S = TPShape<D, Q>;
	return (sizeof(TPOps) + 7) / 8 * 8 + (size_t)S::E * (3 * NV * S::N) * sizeof(double);
}

void record_start(dgpu_ctx* c, const char* name)
{
	if (!c->timing)
		return;
	KernelTimer t;
	t.name = name;
	cudaEventCreate(&t.start);
	cudaEventCreate(&t.stop);
	cudaEventRecord(t.start, c->stream);
	c->timers.push_back(t);
}

void record_stop(dgpu_ctx* c)
{
	if (!c->timing)
		return;
	cudaEventRecord(c->timers.back().stop, c->stream);
}

template <int D, int Q, int NV, int PDE, bool GLL_IN>
cudaError_t launch_volume_t(dgpu_ctx* c)
{
	using S = TPShape<D, Q>;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	record_start(c, "tp_volume_kernel");
	tp_volume_kernel<D, Q, NV, PDE, GLL_IN><<<blocks, S::THREADS, volume_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, c->params(), GLL_IN ? c->u : c->ug);
	record_stop(c);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV, int PDE, int FLUX>
cudaError_t launch_face_t(dgpu_ctx* c)
{
	using S = TPShape<D, Q>;
	const long long n = (long long)c->n_face * S::NF;
	const int blocks = (int)((n + 255) / 256);
	record_start(c, "tp_face_kernel");
	tp_face_kernel<D, Q, NV, PDE, FLUX><<<blocks, 256, 0, c->stream>>>(c->params());
	record_stop(c);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV>
cudaError_t launch_lift_rhs_t(dgpu_ctx* c)
{
	using S = TPShape<D, Q>;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	RkArgs rk;
	rk.u = c->u;
	rk.u0 = c->u0;
	rk.rhs = c->rhs;
	rk.dt = 0.0;
	rk.stage = 0;
	rk.positivity = 0;
	rk.want_max = 1;
	record_start(c, "tp_lift_kernel");
	tp_lift_kernel<D, Q, NV, kModeRhs><<<blocks, S::THREADS, lift_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, c->params(), rk);
	record_stop(c);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV>
cudaError_t launch_lift_rk_t(dgpu_ctx* c, double dt, int stage, int want_max)
{
	using S = TPShape<D, Q>;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	RkArgs rk;
	rk.u = c->ug;
	rk.u0 = c->u0;
	rk.rhs = c->rhs;
	rk.dt = dt;
	rk.stage = stage;
	rk.positivity = c->positivity;
	rk.want_max = want_max;
	record_start(c, "tp_lift_kernel");
	if (want_max)
		tp_lift_kernel<D, Q, NV, kModeRkGl><<<blocks, S::THREADS, lift_smem_bytes<D, Q, NV>(), c->stream>>>(
			c->ops, c->params(), rk);
	else
		tp_lift_kernel<D, Q, NV, kModeRkGlNoMax><<<blocks, S::THREADS, lift_smem_bytes<D, Q, NV>(), c->stream>>>(
			c->ops, c->params(), rk);
	record_stop(c);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV, int PDE>
cudaError_t launch_volume_in_t(dgpu_ctx* c, const double* in, double* keep_coef)
{
	using S = TPShape<D, Q>;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	TPParams P = c->params();
	P.keep_coef = keep_coef;
	P.keep_gl = c->ug;
	tp_volume_kernel<D, Q, NV, PDE, true><<<blocks, S::THREADS, volume_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops,
	                                                                                                      P, in);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV>
cudaError_t launch_lift_out_t(dgpu_ctx* c, double dt, int want_max, double* out_host)
{
	using S = TPShape<D, Q>;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	RkArgs rk;
	rk.u = c->ug;
	rk.u0 = c->u0;
	rk.rhs = c->rhs;
	rk.dt = dt;
	rk.stage = 2;
	rk.positivity = c->positivity;
	rk.want_max = want_max;
	rk.out_coef = c->u;
	rk.out_host = out_host;
	tp_lift_kernel<D, Q, NV, kModeRkGlOut><<<blocks, S::THREADS, lift_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, c->params(), rk);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV>
cudaError_t launch_convert_t(dgpu_ctx* c, bool to_gl, const double* in, double* out, double* in_copy,
                             double* out_copy)
{
	using S = TPShape<D, Q>;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	record_start(c, "tp_convert_kernel");
	if (to_gl)
		tp_convert_kernel<D, Q, NV, true><<<blocks, S::THREADS, convert_smem_bytes<D, Q, NV>(), c->stream>>>(
			c->ops, c->n_vol, in, out, in_copy, out_copy);
	else
		tp_convert_kernel<D, Q, NV, false><<<blocks, S::THREADS, convert_smem_bytes<D, Q, NV>(), c->stream>>>(
			c->ops, c->n_vol, in, out, in_copy, out_copy);
	record_stop(c);
	c->launches++;
	return cudaGetLastError();
}

// VJP of the residual at state u (GLL): 3 kernels (volume + traces, faces, lift + V^T).
template <int D, int Q, int NV, int PDE, int FLUX>
cudaError_t launch_adjoint_t(dgpu_ctx* c, const double* u, const double* rbar, double* ubar)
{
	using S = TPShape<D, Q>;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	AdjArgs A;
	A.u = u;
	A.rbar = rbar;
	A.ubar = ubar;
	A.atraces = c->atraces;
	A.wbar = c->wbar;
	record_start(c, "tp_adj_volume_kernel");
	tp_adj_volume_kernel<D, Q, NV, PDE><<<blocks, S::THREADS, adj_volume_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, c->params(), A);
	record_stop(c);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess)
		return e;
	const long long nfn = (long long)c->n_face * S::NF;
	record_start(c, "tp_adj_face_kernel");
	tp_adj_face_kernel<D, Q, NV, PDE, FLUX><<<(unsigned)((nfn + 127) / 128), 128, 0, c->stream>>>(c->params(), A);
	record_stop(c);
	if ((e = cudaGetLastError()) != cudaSuccess)
		return e;
	record_start(c, "tp_adj_lift_kernel");
	tp_adj_lift_kernel<D, Q, NV><<<blocks, S::THREADS, convert_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, c->params(), A);
	record_stop(c);
	c->launches += 3;
	return cudaGetLastError();
}

// Objective contributions and, when ubar != nullptr, dJ/du = V^T E^T (w_f J_f dp/dW) (vol_gl and wbar are
// zeroed first so that tp_adj_lift_kernel applies the objective's trace cotangent alone).
template <int D, int Q, int NV>
cudaError_t launch_objective_t(dgpu_ctx* c, double* ubar)
{
	using S = TPShape<D, Q>;
	cudaError_t e;
	if (ubar) {
		if ((e = cudaMemsetAsync(c->wbar, 0, (size_t)c->n_face * 2 * NV * S::NF * sizeof(double), c->stream)))
			return e;
		if ((e = cudaMemsetAsync(c->vol_gl, 0, (size_t)c->n_vol * NV * S::N * sizeof(double), c->stream)))
			return e;
	}
	const long long n = (long long)c->n_obj * S::NF;
	tp_objective_kernel<D, S::NF, NV><<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(
		c->params(), c->obj_faces, c->n_obj, c->obj_contrib, c->wbar);
	c->launches++;
	if ((e = cudaGetLastError()) != cudaSuccess || !ubar)
		return e;
	AdjArgs A;
	A.u = nullptr;
	A.rbar = nullptr;
	A.ubar = ubar;
	A.atraces = c->atraces;
	A.wbar = c->wbar;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	tp_adj_lift_kernel<D, Q, NV><<<blocks, S::THREADS, convert_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, c->params(), A);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV>
size_t jvp_volume_smem_bytes()
{
	using S = TPShape<D, Q>;
	return (sizeof(TPOps) + 7) / 8 * 8 + (size_t)S::E * 2 * TPSmem<D, Q, NV>::VOL * sizeof(double);
}

// R(u) and the directional derivative along jv_du: tangent-carrying volume and face kernels, then the residual-mode
// lift on the primal buffers and on the tangent buffers (the lift is linear).
// PRIMAL = false: the derivative only (the primal volume and face quantities are still formed, the primal lift is
// skipped and rhs is left as it was).
template <int D, int Q, int NV, int PDE, int FLUX, bool PRIMAL>
cudaError_t launch_jvp_t(dgpu_ctx* c)
{
	using S = TPShape<D, Q>;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	const TPParams P = c->params();
	TPParams Pd = P;
	Pd.vol_gl = c->jv_vol;
	Pd.traces = c->jv_traces;
	Pd.nnf = c->jv_nnf;
	Pd.source = nullptr;   // the source does not depend on the state
	Pd.max_bits = nullptr;
	cudaError_t e = PRIMAL ? cudaMemsetAsync(c->max_bits, 0, sizeof(unsigned long long), c->stream) : cudaSuccess;
	if (e != cudaSuccess)
		return e;
	tp_jvp_volume_kernel<D, Q, NV, PDE><<<blocks, S::THREADS, jvp_volume_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, P, Pd, c->u, c->jv_du);
	const long long nf = (long long)c->n_face * S::NF;
	tp_jvp_face_kernel<D, Q, NV, PDE, FLUX><<<(unsigned)((nf + 255) / 256), 256, 0, c->stream>>>(P, Pd);
	RkArgs rk;
	rk.u = c->u;
	rk.u0 = c->u0;
	rk.rhs = c->rhs;
	rk.dt = 0.0;
	rk.stage = 0;
	rk.positivity = 0;
	rk.want_max = 1;
	if (PRIMAL)
		tp_lift_kernel<D, Q, NV, kModeRhs><<<blocks, S::THREADS, lift_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, P,
		                                                                                                   rk);
	rk.rhs = c->jv_out;
	tp_lift_kernel<D, Q, NV, kModeRhs><<<blocks, S::THREADS, lift_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, Pd, rk);
	c->launches += PRIMAL ? 4 : 3;
	return cudaGetLastError();
}

template <int D, int Q, int NV>
cudaError_t launch_mass_t(dgpu_ctx* c, const double* in, double* out)
{
	using S = TPShape<D, Q>;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	tp_mass_kernel<D, Q, NV><<<blocks, S::THREADS, lift_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, c->params(), in,
	                                                                                       out);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV, int PDE, int FLUX>
cudaError_t bind(dgpu_ctx* c)
{
	c->launch_adjoint = launch_adjoint_t<D, Q, NV, PDE, FLUX>;
	c->launch_objective = launch_objective_t<D, Q, NV>;
	c->launch_jvp = launch_jvp_t<D, Q, NV, PDE, FLUX, true>;
	c->launch_jvp_tangent = launch_jvp_t<D, Q, NV, PDE, FLUX, false>;
	c->launch_mass = launch_mass_t<D, Q, NV>;
	c->launch_volume = launch_volume_t<D, Q, NV, PDE, true>;
	c->launch_volume_gl = launch_volume_t<D, Q, NV, PDE, false>;
	c->launch_face = launch_face_t<D, Q, NV, PDE, FLUX>;
	c->launch_lift_rhs = launch_lift_rhs_t<D, Q, NV>;
	c->launch_lift_rk = launch_lift_rk_t<D, Q, NV>;
	c->launch_convert = launch_convert_t<D, Q, NV>;
	c->launch_volume_in = launch_volume_in_t<D, Q, NV, PDE>;
	c->launch_lift_out = launch_lift_out_t<D, Q, NV>;
	const cudaFuncAttribute smem = cudaFuncAttributeMaxDynamicSharedMemorySize;
	cudaError_t e;
	if ((e = cudaFuncSetAttribute(tp_lift_kernel<D, Q, NV, kModeRkGlOut>, smem, (int)lift_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_volume_kernel<D, Q, NV, PDE, true>, smem, (int)volume_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_volume_kernel<D, Q, NV, PDE, false>, smem, (int)volume_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_lift_kernel<D, Q, NV, kModeRhs>, smem, (int)lift_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_lift_kernel<D, Q, NV, kModeRkGl>, smem, (int)lift_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_lift_kernel<D, Q, NV, kModeRkGlNoMax>, smem, (int)lift_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_convert_kernel<D, Q, NV, true>, smem, (int)convert_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_adj_volume_kernel<D, Q, NV, PDE>, smem, (int)adj_volume_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_adj_lift_kernel<D, Q, NV>, smem, (int)convert_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_mass_kernel<D, Q, NV>, smem, (int)lift_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_jvp_volume_kernel<D, Q, NV, PDE>, smem, (int)jvp_volume_smem_bytes<D, Q, NV>())))
		return e;
	return cudaFuncSetAttribute(tp_convert_kernel<D, Q, NV, false>, smem, (int)convert_smem_bytes<D, Q, NV>());
}

template <int D, int Q, int NV>
size_t ns_smem_bytes()
{
	using S = TPShape<D, Q>;
	return (sizeof(TPOps) + 7) / 8 * 8 + (size_t)S::E * NsSmem<D, Q, NV>::PER_E * sizeof(double);
}

// Navier-Stokes volume and face work of one residual: gradients and traces, face fluxes, volume flux (the lift that
// follows is the ordinary one).
template <int D, int Q, int FLUX, bool GLL_IN>
cudaError_t launch_ns_t(dgpu_ctx* c)
{
	using S = TPShape<D, Q>;
	constexpr int NV = D + 2;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	const TPParams P = c->params();
	const double* u = GLL_IN ? c->u : c->ug;
	record_start(c, "tp_ns_grad_kernel");
	tp_ns_grad_kernel<D, Q, NV, GLL_IN><<<blocks, S::THREADS, ns_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, P, u);
	record_stop(c);
	const long long nf = (long long)c->n_face * S::NF;
	record_start(c, "tp_ns_face_kernel");
	tp_ns_face_kernel<D, Q, FLUX><<<(unsigned)((nf + 127) / 128), 128, 0, c->stream>>>(P);
	record_stop(c);
	record_start(c, "tp_ns_volume_kernel");
	tp_ns_volume_kernel<D, Q, NV, GLL_IN><<<blocks, S::THREADS, ns_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, P, u);
	record_stop(c);
	c->launches += 3;
	return cudaGetLastError();
}

template <int D, int Q, int NV>
size_t ns_adj_smem_bytes()
{
	using S = TPShape<D, Q>;
	return (sizeof(TPOps) + 7) / 8 * 8 + (size_t)S::E * NsAdjSmem<D, Q, NV>::PER_E * sizeof(double);
}

template <int D, int Q, int NV>
size_t ns_jvp_smem_bytes()
{
	using S = TPShape<D, Q>;
	return (sizeof(TPOps) + 7) / 8 * 8 + (size_t)S::E * NsJvpSmem<D, Q, NV>::PER_E * sizeof(double);
}

// Navier-Stokes R(u) (when PRIMAL) and (dR/du) jv_du: the gradient kernel on u and on du (it is linear), the face and
// volume kernels on dual numbers, the residual-mode lift on the primal and the tangent buffers.
template <int D, int Q, int FLUX, bool PRIMAL>
cudaError_t launch_ns_jvp_t(dgpu_ctx* c)
{
	using S = TPShape<D, Q>;
	constexpr int NV = D + 2;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	const TPParams P = c->params();
	TPParams Pd = P;
	Pd.vol_gl = c->jv_vol;
	Pd.traces = c->jv_traces;
	Pd.nnf = c->jv_nnf;
	Pd.ns_gtr = c->ns_gtr_d;
	Pd.ns_X = c->ns_X_d;
	Pd.ns_gv = c->ns_gv_d;
	Pd.source = nullptr;
	Pd.max_bits = nullptr;
	cudaError_t e = PRIMAL ? cudaMemsetAsync(c->max_bits, 0, sizeof(unsigned long long), c->stream) : cudaSuccess;
	if (e != cudaSuccess)
		return e;
	tp_ns_grad_kernel<D, Q, NV, true><<<blocks, S::THREADS, ns_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, P, c->u);
	tp_ns_grad_kernel<D, Q, NV, true><<<blocks, S::THREADS, ns_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, Pd,
	                                                                                               c->jv_du);
	const long long nf = (long long)c->n_face * S::NF;
	tp_ns_jvp_face_kernel<D, Q, FLUX><<<(unsigned)((nf + 127) / 128), 128, 0, c->stream>>>(P, Pd);
	tp_ns_jvp_volume_kernel<D, Q, NV><<<blocks, S::THREADS, ns_jvp_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, P, Pd, c->u, c->jv_du);
	RkArgs rk;
	rk.u = c->u;
	rk.u0 = c->u0;
	rk.rhs = c->rhs;
	rk.dt = 0.0;
	rk.stage = 0;
	rk.positivity = 0;
	rk.want_max = 1;
	if (PRIMAL)
		tp_lift_kernel<D, Q, NV, kModeRhs><<<blocks, S::THREADS, lift_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, P,
		                                                                                                   rk);
	rk.rhs = c->jv_out;
	tp_lift_kernel<D, Q, NV, kModeRhs><<<blocks, S::THREADS, lift_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, Pd, rk);
	c->launches += PRIMAL ? 6 : 5;
	return cudaGetLastError();
}

// VJP of the Navier-Stokes residual at state u (GLL): the forward gradient and face kernels at u (traces, gradient
// traces, volume gradients, X), then the three adjoint kernels of dgpu_ns_adjoint.cuh.
template <int D, int Q, int FLUX>
cudaError_t launch_ns_adjoint_t(dgpu_ctx* c, const double* u, const double* rbar, double* ubar)
{
	using S = TPShape<D, Q>;
	constexpr int NV = D + 2;
	const int blocks = (c->n_vol + S::E - 1) / S::E;
	const TPParams P = c->params();
	const long long nfn = (long long)c->n_face * S::NF;
	tp_ns_grad_kernel<D, Q, NV, true><<<blocks, S::THREADS, ns_smem_bytes<D, Q, NV>(), c->stream>>>(c->ops, P, u);
	tp_ns_face_kernel<D, Q, FLUX><<<(unsigned)((nfn + 127) / 128), 128, 0, c->stream>>>(P);
	AdjArgs A;
	A.u = u;
	A.rbar = rbar;
	A.ubar = ubar;
	A.atraces = c->atraces;
	A.wbar = c->wbar;
	NsAdjArgs B;
	B.gbar = c->ns_gbar;
	B.xbar = c->ns_xbar;
	B.gtbar = c->ns_gtbar;
	record_start(c, "tp_ns_adj_volume_kernel");
	tp_ns_adj_volume_kernel<D, Q, NV><<<blocks, S::THREADS, ns_adj_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, P, A, B);
	record_stop(c);
	record_start(c, "tp_ns_adj_face_kernel");
	tp_ns_adj_face_kernel<D, Q, FLUX><<<(unsigned)((nfn + 127) / 128), 128, 0, c->stream>>>(P, A, B);
	record_stop(c);
	record_start(c, "tp_ns_adj_lift_kernel");
	tp_ns_adj_lift_kernel<D, Q, NV><<<blocks, S::THREADS, ns_adj_smem_bytes<D, Q, NV>(), c->stream>>>(
		c->ops, P, A, B);
	record_stop(c);
	c->launches += 5;
	return cudaGetLastError();
}

cudaError_t launch_nothing(dgpu_ctx*) { return cudaSuccess; }

template <int D, int Q, int FLUX>
cudaError_t bind_ns(dgpu_ctx* c)
{
	constexpr int NV = D + 2;
	cudaError_t e = bind<D, Q, NV, kEuler, FLUX>(c);   // lift, convert, positivity: as for Euler
	c->launch_volume_in = nullptr;   // the fused host step is Euler / advection only
	c->launch_lift_out = nullptr;
	if (e != cudaSuccess)
		return e;
	c->launch_volume = launch_ns_t<D, Q, FLUX, true>;
	c->launch_volume_gl = launch_ns_t<D, Q, FLUX, false>;
	c->launch_face = launch_nothing;
	c->launch_adjoint = launch_ns_adjoint_t<D, Q, FLUX>;
	c->launch_objective = launch_objective_t<D, Q, NV>;
	c->launch_jvp = launch_ns_jvp_t<D, Q, FLUX, true>;
	c->launch_jvp_tangent = launch_ns_jvp_t<D, Q, FLUX, false>;
	const cudaFuncAttribute smem = cudaFuncAttributeMaxDynamicSharedMemorySize;
	if ((e = cudaFuncSetAttribute(tp_ns_jvp_volume_kernel<D, Q, NV>, smem, (int)ns_jvp_smem_bytes<D, Q, NV>())))
		return e;
	if ((e = cudaFuncSetAttribute(tp_ns_adj_volume_kernel<D, Q, NV>, smem, (int)ns_adj_smem_bytes<D, Q, NV>())) ||
	    (e = cudaFuncSetAttribute(tp_ns_adj_lift_kernel<D, Q, NV>, smem, (int)ns_adj_smem_bytes<D, Q, NV>())))
		return e;
	const int bytes = (int)ns_smem_bytes<D, Q, NV>();
	if ((e = cudaFuncSetAttribute(tp_ns_grad_kernel<D, Q, NV, true>, smem, bytes)) ||
	    (e = cudaFuncSetAttribute(tp_ns_grad_kernel<D, Q, NV, false>, smem, bytes)) ||
	    (e = cudaFuncSetAttribute(tp_ns_volume_kernel<D, Q, NV, true>, smem, bytes)) ||
	    (e = cudaFuncSetAttribute(tp_ns_volume_kernel<D, Q, NV, false>, smem, bytes)))
		return e;
	return cudaSuccess;
}

template <int D, int Q>
cudaError_t bind_pde(dgpu_ctx* c)
{
	if (c->pde == DGPU_PDE_NAVIER_STOKES)
		return c->flux == DGPU_NUM_FLUX_ROE_PIKE ? bind_ns<D, Q, kRoePike>(c) : bind_ns<D, Q, kLaxFriedrichs>(c);
	if (c->pde == DGPU_PDE_ADVECTION)
		return bind<D, Q, 1, kAdvection, kUpwind>(c);
	if (c->flux == DGPU_NUM_FLUX_ROE_PIKE)
		return bind<D, Q, D + 2, kEuler, kRoePike>(c);
	return bind<D, Q, D + 2, kEuler, kLaxFriedrichs>(c);
}

template <int D>
cudaError_t bind_q(dgpu_ctx* c)
{
	switch (c->q) {
	case 2: return bind_pde<D, 2>(c);
	case 3: return bind_pde<D, 3>(c);
	case 4: return bind_pde<D, 4>(c);
	case 5: return bind_pde<D, 5>(c);
	default: return cudaErrorInvalidValue;
	}
}

// Drops the captured step graphs (they hold the kernels' parameters by value: a stream or a buffer that changes makes
// them stale); the next step captures again.
void discard_graphs(dgpu_ctx* c)
{
	if (c->rk_graph) {
		cudaGraphExecDestroy(c->rk_graph);
		c->rk_graph = nullptr;
	}
	if (c->rk_graph_max) {
		cudaGraphExecDestroy(c->rk_graph_max);
		c->rk_graph_max = nullptr;
	}
	if (c->host_graph) {
		cudaGraphExecDestroy(c->host_graph);
		c->host_graph = nullptr;
	}
}

void free_all(dgpu_ctx* c)
{
	discard_graphs(c);
	for (auto& t : c->timers) {
		cudaEventDestroy(t.start);
		cudaEventDestroy(t.stop);
	}
	c->timers.clear();
	void* ptrs[] = {c->source, c->halo_send, c->halo_recv, c->halo_sbuf, c->halo_rbuf, c->jv_du, c->jv_vol, c->jv_traces, c->jv_nnf, c->jv_out, c->obj_faces, c->obj_contrib, c->u_saved, c->vbar, c->ubar, c->atraces, c->wbar, c->u, c->u0, c->ug, c->rhs, c->gmet, c->inv_wJ, c->fgeo, c->vol_face, c->nc, c->nc_inv,
	                c->jac_slot, c->jac_members, c->ns_gtr, c->ns_lam, c->ns_X, c->ns_gv, c->ns_gtr_d, c->ns_X_d, c->ns_gv_d, c->ns_gbar, c->ns_xbar, c->ns_gtbar,
	                c->bnd, c->bc_code, c->bc_ext, c->traces, c->nnf, c->vol_gl, c->max_bits, c->err_flag, c->n_corr};
	for (void* p : ptrs)
		if (p)
			cudaFree(p);
	if (c->own_stream && c->stream)
		cudaStreamDestroy(c->stream);
}

template <typename T>
cudaError_t upload(T** dst, const std::vector<T>& src)
{
	cudaError_t e = cudaMalloc((void**)dst, src.size() * sizeof(T));
	if (e != cudaSuccess)
		return e;
	return cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
}

size_t state_size(const dgpu_ctx* c) { return (size_t)c->n_vol * c->nv * c->N; }

// The geometry operators of a QUAD/HEX element of order p with geometry order p_g (the TP factors of the
// reference's cv1_vg_vm, cv1_vg_vc, vv0_vm_vc and vv0_vm_fc), derived from their GLL and GL node sets, and the
// reference normals of its local faces (element.c:708-780, with the same cos/sin round-off).
void build_geo_ops(int d, int q, int p_g, const double* w_vc, GeoOps* G)
{
	memset(G, 0, sizeof *G);
	G->d = d;
	G->qg = p_g + 1;
	G->q = q;
	double xg[kQMax], xc[kQMax];
	gauss_lobatto_nodes(G->qg, xg);
	gauss_legendre_nodes(q, xc);
	for (int a = 0; a < G->qg; ++a) {
		for (int m = 0; m < G->qg; ++m)
			G->Dgg[m][a] = lagrange_derivative(xg, G->qg, a, xg[m]);
		for (int c = 0; c < q; ++c) {
			G->Lgc[c][a] = lagrange_value(xg, G->qg, a, xc[c]);
			G->Dgc[c][a] = lagrange_derivative(xg, G->qg, a, xc[c]);
		}
		G->Lgb[0][a] = lagrange_value(xg, G->qg, a, -1.0);
		G->Lgb[1][a] = lagrange_value(xg, G->qg, a, 1.0);
	}
	const double t_z[6] = {M_PI, 0.0, 1.5 * M_PI, 0.5 * M_PI, 0.0, M_PI};
	const double t_e[6] = {0.0, 0.0, 0.0, 0.0, 0.5 * M_PI, 1.5 * M_PI};
	for (int lf = 0; lf < 2 * d; ++lf) {
		G->nref[lf][0] = cos(t_e[lf]) * cos(t_z[lf]);
		G->nref[lf][1] = cos(t_e[lf]) * sin(t_z[lf]);
		G->nref[lf][2] = (d == 3 ? -sin(t_e[lf]) : 0.0);
	}
	for (int c = 0; c < q; ++c)
		G->w[c] = w_vc[c];
}

// Volume then face geometry on the stream; out.metrics_vm and out.err must be device buffers (n_vol d^2 n_g doubles,
// one int set to 0).
cudaError_t run_geometry(const GeoOps& G, int n_vol, int n_face, const double* geom_coef, const int* face_vol,
                         const int* face_lf, const GeoOut& out, cudaStream_t st)
{
	const size_t smem = kGeoSmem * sizeof(double);
	cudaError_t e = cudaFuncSetAttribute(geo_volume_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess)
		return e;
	geo_volume_kernel<<<(unsigned)n_vol, 128, smem, st>>>(G, n_vol, geom_coef, out);
	if ((e = cudaGetLastError()) != cudaSuccess)
		return e;
	const int nf = (G.d == 2 ? G.q : G.q * G.q);
	const long long n_nodes = (long long)n_face * nf;
	if (n_nodes > 0)
		geo_face_kernel<<<(unsigned)((n_nodes + 127) / 128), 128, 0, st>>>(G, n_face, face_vol, face_lf, geom_coef,
		                                                                   out);
	return cudaGetLastError();
}

// Device buffers of one geometry computation: the coefficients and side-0 connectivity copied in, the vm metric
// scratch and the error flag. The connectivity must have been checked on the host (side 0 in range).
struct GeoBuffers {
	double* geom = nullptr;
	double* mvm = nullptr;
	int* fv = nullptr;
	int* flf = nullptr;
	int* err = nullptr;
	~GeoBuffers()
	{
		void* ptrs[] = {geom, mvm, fv, flf, err};
		for (void* p : ptrs)
			if (p)
				cudaFree(p);
	}
	cudaError_t init(const dgpu_mesh* m, int d, cudaStream_t st)
	{
		const int qg = m->p_g + 1;
		const size_t ng = (d == 2 ? qg * qg : qg * qg * qg), nv = (size_t)m->n_volumes, nf = (size_t)m->n_faces;
		cudaError_t e;
		if ((e = cudaMalloc((void**)&geom, nv * ng * d * sizeof(double))) ||
		    (e = cudaMalloc((void**)&mvm, nv * ng * d * d * sizeof(double))) ||
		    (e = cudaMalloc((void**)&fv, (nf > 0 ? nf : 1) * 2 * sizeof(int))) ||
		    (e = cudaMalloc((void**)&flf, (nf > 0 ? nf : 1) * 2 * sizeof(int))) ||
		    (e = cudaMalloc((void**)&err, sizeof(int))))
			return e;
		if ((e = cudaMemcpyAsync(geom, m->geom_coef, nv * ng * d * sizeof(double), cudaMemcpyHostToDevice, st)) ||
		    (nf > 0 && (e = cudaMemcpyAsync(fv, m->face_vol, nf * 2 * sizeof(int), cudaMemcpyHostToDevice, st))) ||
		    (nf > 0 && (e = cudaMemcpyAsync(flf, m->face_lf, nf * 2 * sizeof(int), cudaMemcpyHostToDevice, st))))
			return e;
		return cudaMemsetAsync(err, 0, sizeof(int), st);
	}
	// Runs the kernels into `out` (whose metrics_vm and err are set here) and returns the error flag.
	cudaError_t run(const GeoOps& G, const dgpu_mesh* m, GeoOut out, cudaStream_t st, int* h_err)
	{
		out.metrics_vm = mvm;
		out.err = err;
		cudaError_t e = run_geometry(G, m->n_volumes, m->n_faces, geom, fv, flf, out, st);
		if (e != cudaSuccess)
			return e;
		if ((e = cudaMemcpyAsync(h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
			return e;
		return cudaStreamSynchronize(st);
	}
};

// The context's gmet, inv_wJ and fgeo from the mesh's geometry coefficients.
dgpu_status device_geometry(dgpu_ctx* c, const dgpu_tp_operators* ops, const dgpu_mesh* mesh)
{
	GeoOps G;
	build_geo_ops(c->d, c->q, mesh->p_g, ops->w_vc, &G);
	GeoBuffers B;
	GeoOut out = {};
	out.gmet = c->gmet;
	out.inv_wJ = c->inv_wJ;
	out.fgeo = c->fgeo;
	int h_err = 0;
	cudaError_t e = B.init(mesh, c->d, c->stream);
	if (e == cudaSuccess)
		e = B.run(G, mesh, out, c->stream, &h_err);
	if (e != cudaSuccess)
		return cuda_fail(nullptr, e, "device geometry");
	if (h_err)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "non-positive Jacobian determinant (device geometry)");
	return DGPU_OK;
}

// One residual (volume, face, lift) on the stream.
dgpu_status enqueue_rhs(dgpu_ctx* c)
{
	DGPU_CUDA(c, c->launch_volume(c));
	DGPU_CUDA(c, c->launch_face(c));
	DGPU_CUDA(c, c->launch_lift_rhs(c));
	return DGPU_OK;
}

// One SSP-RK3 step on the GL nodal state ug (3 x volume, face, lift); max|rhs| of the last stage on request.
// (Fusing each lift with the next stage's volume term into one kernel was measured slower: the fused kernel runs
// at the lift's 128 registers, which halves the volume term's occupancy.)
dgpu_status enqueue_rk_step(dgpu_ctx* c, double dt, bool want_max)
{
	for (int stage = 0; stage < 3; ++stage) {
		DGPU_CUDA(c, c->launch_volume_gl(c));
		DGPU_CUDA(c, c->launch_face(c));
		DGPU_CUDA(c, c->launch_lift_rk(c, dt, stage, (want_max && stage == 2) ? 1 : 0));
	}
	return DGPU_OK;
}

// Make u (GLL coefficients) current: V^-1 of ug after time stepping.
dgpu_status ensure_coef(dgpu_ctx* c)
{
	if (!c->coef_valid) {
		DGPU_CUDA(c, c->launch_convert(c, false, c->ug, c->u, nullptr, nullptr));
		c->coef_valid = true;
	}
	return DGPU_OK;
}

// Make ug (GL nodal values) current: V u after an upload.
dgpu_status ensure_gl(dgpu_ctx* c)
{
	if (!c->gl_valid) {
		DGPU_CUDA(c, c->launch_convert(c, true, c->u, c->ug, nullptr, nullptr));
		c->gl_valid = true;
	}
	return DGPU_OK;
}

dgpu_status read_max(dgpu_ctx* c, double* max_rhs)
{
	if (!max_rhs)
		return DGPU_OK;
	unsigned long long bits = 0;
	DGPU_CUDA(c, cudaMemcpyAsync(&bits, c->max_bits, sizeof bits, cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	double v;
	memcpy(&v, &bits, sizeof v);
	*max_rhs = v;
	return DGPU_OK;
}

// Entry points that evaluate the whole mesh refuse a partitioned context: its remote traces come only from the
// dgpu_halo_* calls.
#define DGPU_WHOLE_MESH(c)                                                                                        \
	do {                                                                                                          \
		if ((c) && (c)->n_remote > 0)                                                                             \
			return fail((c), DGPU_ERR_INVALID_ARGUMENT,                                                           \
			            "partitioned context: evaluate it with dgpu_halo_stage_begin / dgpu_halo_stage_end");       \
	} while (0)

// Copies trace slots between the trace array and a halo buffer: pack reads traces[slot] into buf[i], unpack writes
// buf[i] into traces[slot]. One thread per double; a slot is nv x NF contiguous doubles of [f][side][var][node].
__global__ void halo_copy_kernel(double* __restrict__ traces, double* __restrict__ buf, const int* __restrict__ slots,
                                 int n, int slot_doubles, int pack)
{
	const long long total = (long long)n * slot_doubles;
	for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
	     idx += (long long)gridDim.x * blockDim.x) {
		const long long i = idx / slot_doubles;
		const long long t = (long long)slots[i] * slot_doubles + (idx - i * slot_doubles);
		if (pack)
			buf[idx] = traces[t];
		else
			traces[t] = buf[idx];
	}
}

cudaError_t launch_halo_copy(dgpu_ctx* c, bool pack)
{
	if (c->n_halo == 0)
		return cudaSuccess;
	const int slot = c->nv * c->NF;
	const long long total = (long long)c->n_halo * slot;
	const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 8);
	halo_copy_kernel<<<blocks, 256, 0, c->stream>>>(c->traces, pack ? c->halo_sbuf : c->halo_rbuf,
	                                                 pack ? c->halo_send : c->halo_recv, c->n_halo, slot, pack ? 1 : 0);
	c->launches++;
	return cudaGetLastError();
}

dgpu_status check_positivity_flag(dgpu_ctx* c)
{
	if (!c->positivity)
		return DGPU_OK;
	int flag = 0;
	DGPU_CUDA(c, cudaMemcpyAsync(&flag, c->err_flag, sizeof flag, cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	if (flag)
		return fail(c, DGPU_ERR_POSITIVITY, "average density or pressure below EPS_PHYS");
	return DGPU_OK;
}

}  // namespace

extern "C" {

const char* dgpu_status_string(dgpu_status st)
{
	switch (st) {
	case DGPU_OK: return "ok";
	case DGPU_ERR_INVALID_ARGUMENT: return "invalid argument";
	case DGPU_ERR_UNSUPPORTED: return "unsupported";
	case DGPU_ERR_CUDA: return "CUDA error";
	case DGPU_ERR_POSITIVITY: return "positivity failure";
	case DGPU_ERR_NO_DEVICE: return "no sm_103 device";
	default: return "unknown status";
	}
}

const char* dgpu_last_error(const dgpu_ctx* ctx)
{
	return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

dgpu_status dgpu_create(const dgpu_physics* phys, const dgpu_tp_operators* ops, const dgpu_mesh* mesh,
                        dgpu_ctx** out)
{
	g_create_error.clear();
	if (!phys || !ops || !mesh || !out)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "NULL argument");
	*out = nullptr;
	const int d = phys->d;
	if (d != 2 && d != 3)
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "d must be 2 or 3");
	if ((d == 2 && ops->elem_type != DGPU_QUAD) || (d == 3 && ops->elem_type != DGPU_HEX))
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "element type must be QUAD (d=2) or HEX (d=3)");
	if (ops->p < 1 || ops->p > kQMax - 1)
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "p must be in 1..4");
	if (phys->pde == DGPU_PDE_ADVECTION) {
		if (phys->num_flux != DGPU_NUM_FLUX_UPWIND)
			return fail(nullptr, DGPU_ERR_UNSUPPORTED, "advection supports the upwind flux");
	} else if (phys->pde == DGPU_PDE_EULER || phys->pde == DGPU_PDE_NAVIER_STOKES) {
		if (phys->num_flux != DGPU_NUM_FLUX_ROE_PIKE && phys->num_flux != DGPU_NUM_FLUX_LAX_FRIEDRICHS)
			return fail(nullptr, DGPU_ERR_UNSUPPORTED, "Euler supports Roe-Pike and Lax-Friedrichs");
		if (phys->pde == DGPU_PDE_NAVIER_STOKES &&
		    ((phys->viscosity != DGPU_VISCOSITY_CONSTANT && phys->viscosity != DGPU_VISCOSITY_SUTHERLAND) ||
		     !(phys->mu >= 0.0) || !(phys->Pr > 0.0) ||
		     (phys->viscosity == DGPU_VISCOSITY_SUTHERLAND && !(phys->r_s > 0.0))))
			return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "Navier-Stokes needs a viscosity model, mu >= 0, Pr > 0"
			                                               " (and r_s > 0 for Sutherland's law)");
		if (phys->pde == DGPU_PDE_NAVIER_STOKES && phys->dTdn != 0.0 && phys->viscosity != DGPU_VISCOSITY_CONSTANT)
			return fail(nullptr, DGPU_ERR_UNSUPPORTED, "a diabatic wall flux (dTdn != 0) needs constant viscosity");
	} else {
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "pde must be advection, Euler or Navier-Stokes");
	}
	if (!ops->cv0_vs_vc || !ops->cv1_vs_vc || !ops->cv0_vs_fc || !ops->w_vc)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "NULL operator");
	if (phys->pde != DGPU_PDE_ADVECTION && phys->positivity && (!ops->ccSB0_vs_vs || !ops->ccBS0_vs_vs))
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "positivity needs ccSB0/ccBS0");
	// geometry: the geometric factors, or the geometry coefficients from which the device computes them
	const bool dev_geo = mesh->geom_coef != nullptr;
	const bool host_geo = mesh->metrics_vc && mesh->jacobian_det_vc && mesh->normals_fc && mesh->jacobian_det_fc;
	if (mesh->n_volumes < 1 || mesh->n_faces < 1 || !mesh->face_vol || !mesh->face_lf || dev_geo == host_geo ||
	    (dev_geo && (mesh->metrics_vc || mesh->jacobian_det_vc || mesh->normals_fc || mesh->jacobian_det_fc)))
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT,
		            "incomplete mesh (give either the four geometric factor arrays or geom_coef)");
	if (dev_geo && (mesh->p_g < 1 || mesh->p_g > kQMax - 1))
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "p_g must be in 1..4");

	int dev = 0, n_dev = 0;
	if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev < 1)
		return fail(nullptr, DGPU_ERR_NO_DEVICE, "no CUDA device");
	cudaGetDevice(&dev);
	cudaDeviceProp prop;
	if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || prop.major * 10 + prop.minor != 103)
		return fail(nullptr, DGPU_ERR_NO_DEVICE, "device is not compute capability 10.3 (sm_103a build)");

	dgpu_ctx* c = new dgpu_ctx();
	c->d = d;
	c->q = ops->p + 1;
	const int q = c->q;
	c->N = (d == 2 ? q * q : q * q * q);
	c->NF = (d == 2 ? q : q * q);
	c->pde = phys->pde;
	c->flux = phys->num_flux;
	c->nv = (phys->pde != DGPU_PDE_ADVECTION ? d + 2 : 1);
	c->positivity = (phys->pde != DGPU_PDE_ADVECTION && phys->positivity) ? 1 : 0;
	c->ns = phys->pde == DGPU_PDE_NAVIER_STOKES;
	if (c->ns) {
		c->ns_phys = NsPhys{phys->mu, phys->Pr, phys->r_s, phys->viscosity,
		                    -phys->mu * (kGamma / kGm1 * phys->r_s) / phys->Pr * phys->dTdn};
		c->stage_launches = 4;
	}
	c->n_vol = mesh->n_volumes;
	c->n_face = mesh->n_faces;
	for (int k = 0; k < 3; ++k)
		c->b_adv[k] = phys->b_adv[k];
	const int N = c->N, NF = c->NF;

	// ---- 1D operators: B, B^-1, GL collocation derivative, GL boundary values, positivity maps ----
	if (!derive_tp_ops(ops, d, &c->ops)) {
		delete c;
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "cv0_vs_vc is singular");
	}

	// ---- weights: TP products of the 1D GL rule (first direction fastest) ----
	std::vector<double> w(N), wf(NF);
	for (int n = 0; n < N; ++n) {
		int r = n;
		double x = 1.0;
		for (int k = 0; k < d; ++k) {
			x *= ops->w_vc[r % q];
			r /= q;
		}
		w[n] = x;
	}
	for (int n = 0; n < NF; ++n) {
		int r = n;
		double x = 1.0;
		for (int k = 0; k < d - 1; ++k) {
			x *= ops->w_vc[r % q];
			r /= q;
		}
		wf[n] = x;
	}

	// ---- volume geometry ----
	const size_t nV = (size_t)c->n_vol;
	std::vector<double> gmet(dev_geo ? 0 : nV * d * d * N), inv_wJ(dev_geo ? 0 : nV * N);
	for (size_t v = 0; v < (dev_geo ? 0 : nV); ++v) {
		const double* m = mesh->metrics_vc + v * (size_t)N * d * d;
		const double* J = mesh->jacobian_det_vc + v * (size_t)N;
		for (int j = 0; j < d; ++j)
			for (int i = 0; i < d; ++i)
				for (int n = 0; n < N; ++n)
					gmet[((v * d + j) * d + i) * N + n] = w[n] * m[n + (size_t)N * (i + d * j)];
		for (int n = 0; n < N; ++n) {
			if (!(J[n] > 0.0)) {
				delete c;
				return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "non-positive jacobian_det_vc");
			}
			inv_wJ[v * N + n] = 1.0 / (w[n] * J[n]);
		}
	}

	// ---- faces ----
	const size_t nF = (size_t)c->n_face;
	std::vector<double> fgeo(dev_geo ? 0 : nF * (d + 1) * NF);
	std::vector<int> vol_face(nV * 2 * d, -1);
	bool any_perm = false;
	std::vector<int> nc, nc_inv;
	if (mesh->nc_fc) {
		nc.assign(mesh->nc_fc, mesh->nc_fc + nF * NF);
		nc_inv.assign(nF * NF, -1);
	}
	// boundary faces: side 1 absent; their BC code and exterior state, compacted to the boundary list
	std::vector<int> bnd(nF, -1), bc_code;
	std::vector<double> bc_ext;
	int n_remote = 0;
	for (size_t f = 0; f < nF; ++f) {
		const bool rem0 = mesh->face_vol[2 * f] == DGPU_REMOTE_VOLUME;
		const bool rem1 = mesh->face_vol[2 * f + 1] == DGPU_REMOTE_VOLUME;
		if (rem0 && rem1) {
			delete c;
			return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "a face with both sides on other ranks");
		}
		const bool boundary = mesh->face_vol[2 * f + 1] < 0 && !rem1;
		for (int s = 0; s < (boundary ? 1 : 2); ++s) {
			if ((s == 0 && rem0) || (s == 1 && rem1)) {   // the other rank's side: its trace arrives by exchange
				++n_remote;
				continue;
			}
			const int v = mesh->face_vol[2 * f + s], lf = mesh->face_lf[2 * f + s];
			if (v < 0 || v >= c->n_vol || lf < 0 || lf >= 2 * d || vol_face[(size_t)v * 2 * d + lf] != -1) {
				delete c;
				return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "bad face connectivity");
			}
			vol_face[(size_t)v * 2 * d + lf] = (int)(2 * f + s);
		}
		if (boundary) {
			if (!mesh->bc_fc || !mesh->bc_state_fc) {
				delete c;
				return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "boundary faces need bc_fc and bc_state_fc");
			}
			const int code = mesh->bc_fc[f] % kBcStepSC;
			if (code < 0 || (c->ns ? !bc_is_navier_stokes(code)
			                       : (c->pde == DGPU_PDE_EULER ? !bc_is_euler(code) : !bc_is_advection_upwind(code)))) {
				delete c;
				return fail(nullptr, DGPU_ERR_UNSUPPORTED,
				            "BC code " + std::to_string(mesh->bc_fc[f]) + " is not provided for this pde");
			}
			if ((code == kBcBackPressure || code == kBcTotalTP) && !mesh->bc_data) {
				delete c;
				return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "back pressure / total TP faces need bc_data");
			}
			bnd[f] = (int)bc_code.size();
			bc_code.push_back(code);
			const double* e = mesh->bc_state_fc + f * (size_t)NF * c->nv;
			for (int k = 0; k < c->nv; ++k)
				for (int i = 0; i < NF; ++i)
					bc_ext.push_back(e[(size_t)i * c->nv + k]);
		}
		for (int i = 0; i < (dev_geo ? 0 : NF); ++i) {
			for (int k = 0; k < d; ++k)
				fgeo[(f * (d + 1) + k) * NF + i] = mesh->normals_fc[(f * NF + i) * d + k];
			fgeo[(f * (d + 1) + d) * NF + i] = wf[i] * mesh->jacobian_det_fc[f * NF + i];
		}
		if (mesh->nc_fc && !boundary) {
			for (int i = 0; i < NF; ++i) {
				const int t = nc[f * NF + i];
				if (t < 0 || t >= NF || nc_inv[f * NF + t] != -1) {
					delete c;
					return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "nc_fc is not a permutation");
				}
				nc_inv[f * NF + t] = i;
				if (t != i)
					any_perm = true;
			}
		}
	}
	c->h_face_vol.assign(mesh->face_vol, mesh->face_vol + 2 * nF);
	c->n_remote = n_remote;
	if (n_remote > 0 && c->ns) {
		delete c;
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "partitioned meshes: Euler and advection only");
	}
	for (size_t i = 0; i < vol_face.size(); ++i)
		if (vol_face[i] < 0) {
			delete c;
			return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "a volume face is missing from the face list");
		}

	// ---- device allocations ----
	const size_t ns = state_size(c);
#define DG_TRY(call)                                        \
	do {                                                    \
		cudaError_t e_ = (call);                            \
		if (e_ != cudaSuccess) {                            \
			std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_); \
			free_all(c);                                    \
			delete c;                                       \
			return fail(nullptr, DGPU_ERR_CUDA, m_);        \
		}                                                   \
	} while (0)
	DG_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
	c->own_stream = true;
	DG_TRY(cudaMalloc((void**)&c->u, ns * sizeof(double)));
	DG_TRY(cudaMalloc((void**)&c->u0, ns * sizeof(double)));
	DG_TRY(cudaMalloc((void**)&c->ug, ns * sizeof(double)));
	DG_TRY(cudaMalloc((void**)&c->rhs, ns * sizeof(double)));
	DG_TRY(cudaMalloc((void**)&c->vol_gl, ns * sizeof(double)));
	DG_TRY(cudaMalloc((void**)&c->traces, nF * 2 * c->nv * NF * sizeof(double)));
	DG_TRY(cudaMalloc((void**)&c->nnf, nF * c->nv * NF * sizeof(double)));
	DG_TRY(cudaMalloc((void**)&c->max_bits, sizeof(unsigned long long)));
	DG_TRY(cudaMalloc((void**)&c->err_flag, sizeof(int)));
	DG_TRY(cudaMalloc((void**)&c->n_corr, sizeof(unsigned long long)));
	DG_TRY(cudaMemset(c->u, 0, ns * sizeof(double)));
	DG_TRY(cudaMemset(c->u0, 0, ns * sizeof(double)));
	DG_TRY(cudaMemset(c->rhs, 0, ns * sizeof(double)));
	DG_TRY(cudaMemset(c->max_bits, 0, sizeof(unsigned long long)));
	DG_TRY(cudaMemset(c->err_flag, 0, sizeof(int)));
	DG_TRY(cudaMemset(c->n_corr, 0, sizeof(unsigned long long)));
	if (dev_geo) {
		DG_TRY(cudaMalloc((void**)&c->gmet, nV * d * d * N * sizeof(double)));
		DG_TRY(cudaMalloc((void**)&c->inv_wJ, nV * N * sizeof(double)));
		DG_TRY(cudaMalloc((void**)&c->fgeo, nF * (d + 1) * NF * sizeof(double)));
		const dgpu_status gs = device_geometry(c, ops, mesh);
		if (gs != DGPU_OK) {
			free_all(c);
			delete c;
			return gs;
		}
	} else {
		DG_TRY(upload(&c->gmet, gmet));
		DG_TRY(upload(&c->inv_wJ, inv_wJ));
		DG_TRY(upload(&c->fgeo, fgeo));
	}
	DG_TRY(upload(&c->vol_face, vol_face));
	if (any_perm) {
		for (size_t f = 0; f < nF; ++f)   // boundary faces: unused entries, kept a permutation
			if (bnd[f] >= 0)
				for (int i = 0; i < NF; ++i)
					nc[f * NF + i] = nc_inv[f * NF + i] = i;
		DG_TRY(upload(&c->nc, nc));
		DG_TRY(upload(&c->nc_inv, nc_inv));
	}
	c->n_bnd = (int)bc_code.size();
	if (mesh->bc_data)
		c->bc_data = BcData{mesh->bc_data[0], mesh->bc_data[1], mesh->bc_data[2], mesh->bc_data[3]};
	if (c->n_bnd > 0) {
		DG_TRY(upload(&c->bnd, bnd));
		DG_TRY(upload(&c->bc_code, bc_code));
		DG_TRY(upload(&c->bc_ext, bc_ext));
	}
	if (c->ns) {   // BR2 buffers and the faces' own lifting diagonal
		DG_TRY(cudaMalloc((void**)&c->ns_gtr, nF * 2 * d * c->nv * NF * sizeof(double)));
		DG_TRY(cudaMalloc((void**)&c->ns_lam, nF * 2 * NF * sizeof(double)));
		DG_TRY(cudaMalloc((void**)&c->ns_X, nF * d * c->nv * NF * sizeof(double)));
		DG_TRY(cudaMalloc((void**)&c->ns_gv, nV * d * c->nv * N * sizeof(double)));
		const long long n_lam = (long long)nV * 2 * d * NF;
		const unsigned g = (unsigned)((n_lam + 255) / 256);
		switch ((d == 2 ? 10 : 20) + q) {
		case 12: tp_ns_lambda_kernel<2, 2><<<g, 256, 0, c->stream>>>(c->ops, c->params(), c->ns_lam); break;
		case 13: tp_ns_lambda_kernel<2, 3><<<g, 256, 0, c->stream>>>(c->ops, c->params(), c->ns_lam); break;
		case 14: tp_ns_lambda_kernel<2, 4><<<g, 256, 0, c->stream>>>(c->ops, c->params(), c->ns_lam); break;
		case 15: tp_ns_lambda_kernel<2, 5><<<g, 256, 0, c->stream>>>(c->ops, c->params(), c->ns_lam); break;
		case 22: tp_ns_lambda_kernel<3, 2><<<g, 256, 0, c->stream>>>(c->ops, c->params(), c->ns_lam); break;
		case 23: tp_ns_lambda_kernel<3, 3><<<g, 256, 0, c->stream>>>(c->ops, c->params(), c->ns_lam); break;
		case 24: tp_ns_lambda_kernel<3, 4><<<g, 256, 0, c->stream>>>(c->ops, c->params(), c->ns_lam); break;
		default: tp_ns_lambda_kernel<3, 5><<<g, 256, 0, c->stream>>>(c->ops, c->params(), c->ns_lam); break;
		}
		DG_TRY(cudaGetLastError());
		DG_TRY(cudaStreamSynchronize(c->stream));
	}
	cudaError_t be = (d == 2 ? bind_q<2>(c) : bind_q<3>(c));
	if (be != cudaSuccess) {
		std::string m_ = std::string("kernel set-up: ") + cudaGetErrorString(be);
		free_all(c);
		delete c;
		return fail(nullptr, DGPU_ERR_CUDA, m_);
	}
#undef DG_TRY
	*out = c;
	return DGPU_OK;
}

dgpu_status dgpu_destroy(dgpu_ctx* ctx)
{
	if (!ctx)
		return DGPU_ERR_INVALID_ARGUMENT;
	if (ctx->stream)
		cudaStreamSynchronize(ctx->stream);
	free_all(ctx);
	delete ctx;
	return DGPU_OK;
}

dgpu_status dgpu_state_size(const dgpu_ctx* ctx, size_t* n)
{
	if (!ctx || !n)
		return DGPU_ERR_INVALID_ARGUMENT;
	*n = state_size(ctx);
	return DGPU_OK;
}

// The device address of a caller's page-locked host buffer (cudaHostAlloc / cudaHostRegister), which kernels may
// read and write directly over the host link; null for any other pointer (pageable or device memory).
double* pinned_device_view(const void* host)
{
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
		cudaGetLastError();
		return nullptr;
	}
	return a.type == cudaMemoryTypeHost ? static_cast<double*>(a.devicePointer) : nullptr;
}

dgpu_status dgpu_upload_state(dgpu_ctx* c, const double* sol)
{
	if (!c || !sol)
		return DGPU_ERR_INVALID_ARGUMENT;
	if (double* dv = c->launch_convert ? pinned_device_view(sol) : nullptr) {
		// a pinned buffer: one pass reads it over the host link, keeps the coefficients and forms the GL values
		DGPU_CUDA(c, c->launch_convert(c, true, dv, c->ug, c->u, nullptr));
		DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
		c->coef_valid = true;
		c->gl_valid = true;
		return DGPU_OK;
	}
	DGPU_CUDA(c, cudaMemcpyAsync(c->u, sol, state_size(c) * sizeof(double), cudaMemcpyHostToDevice, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	c->coef_valid = true;
	c->gl_valid = false;
	return DGPU_OK;
}

dgpu_status dgpu_download_state(dgpu_ctx* c, double* sol)
{
	if (!c || !sol)
		return DGPU_ERR_INVALID_ARGUMENT;
	if (!c->coef_valid && c->launch_convert) {
		if (double* dv = pinned_device_view(sol)) {
			// the coefficients are stale: V^-1 of the GL values written to the device copy and the pinned buffer
			DGPU_CUDA(c, c->launch_convert(c, false, c->ug, c->u, nullptr, dv));
			DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
			c->coef_valid = true;
			return DGPU_OK;
		}
	}
	dgpu_status st = ensure_coef(c);
	if (st != DGPU_OK)
		return st;
	DGPU_CUDA(c, cudaMemcpyAsync(sol, c->u, state_size(c) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}

dgpu_status dgpu_download_rhs(dgpu_ctx* c, double* rhs)
{
	if (!c || !rhs)
		return DGPU_ERR_INVALID_ARGUMENT;
	DGPU_CUDA(c, cudaMemcpyAsync(rhs, c->rhs, state_size(c) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}

dgpu_status dgpu_compute_rhs(dgpu_ctx* c, double* max_rhs)
{
	DGPU_WHOLE_MESH(c);
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	dgpu_status st = ensure_coef(c);
	if (st != DGPU_OK)
		return st;
	st = enqueue_rhs(c);
	if (st != DGPU_OK)
		return st;
	return read_max(c, max_rhs);
}

dgpu_status dgpu_compute_rhs_host(dgpu_ctx* c, const double* sol, double* rhs, double* max_rhs)
{
	DGPU_WHOLE_MESH(c);
	if (!c || !sol || !rhs)
		return DGPU_ERR_INVALID_ARGUMENT;
	const size_t bytes = state_size(c) * sizeof(double);
	DGPU_CUDA(c, cudaMemcpyAsync(c->u, sol, bytes, cudaMemcpyHostToDevice, c->stream));
	c->coef_valid = true;
	c->gl_valid = false;
	dgpu_status st = enqueue_rhs(c);
	if (st != DGPU_OK)
		return st;
	DGPU_CUDA(c, cudaMemcpyAsync(rhs, c->rhs, bytes, cudaMemcpyDeviceToHost, c->stream));
	if (max_rhs)
		return read_max(c, max_rhs);
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}

// Captures one step into *graph (for dt) unless the cached one matches.
static dgpu_status capture_step(dgpu_ctx* c, double dt, bool want_max, cudaGraphExec_t* graph, double* graph_dt)
{
	if (*graph && *graph_dt == dt)
		return DGPU_OK;
	if (*graph) {
		cudaGraphExecDestroy(*graph);
		*graph = nullptr;
	}
	cudaGraph_t g;
	DGPU_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
	const long long before = c->launches;
	dgpu_status st = enqueue_rk_step(c, dt, want_max);
	c->launches = before;  // captured, not launched
	cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
	if (st != DGPU_OK)
		return st;
	DGPU_CUDA(c, ec);
	cudaError_t ei = cudaGraphInstantiate(graph, g, 0);
	cudaGraphDestroy(g);
	DGPU_CUDA(c, ei);
	*graph_dt = dt;
	return DGPU_OK;
}

dgpu_status dgpu_ssp_rk3_steps(dgpu_ctx* c, double dt, int n_steps, double* max_rhs)
{
	DGPU_WHOLE_MESH(c);
	if (!c || n_steps < 0 || !(dt == dt))
		return DGPU_ERR_INVALID_ARGUMENT;
	dgpu_status st = ensure_gl(c);
	if (st != DGPU_OK)
		return st;
	const bool want_max = (max_rhs != nullptr);
	if (c->timing) {
		for (int s = 0; s < n_steps; ++s) {
			st = enqueue_rk_step(c, dt, want_max && s == n_steps - 1);
			if (st != DGPU_OK)
				return st;
		}
	} else {
		const int plain = want_max ? n_steps - 1 : n_steps;
		if (plain > 0 && (st = capture_step(c, dt, false, &c->rk_graph, &c->rk_graph_dt)) != DGPU_OK)
			return st;
		if (want_max && n_steps > 0 &&
		    (st = capture_step(c, dt, true, &c->rk_graph_max, &c->rk_graph_max_dt)) != DGPU_OK)
			return st;
		for (int s = 0; s < plain; ++s) {
			DGPU_CUDA(c, cudaGraphLaunch(c->rk_graph, c->stream));
			c->launches += 3 * c->stage_launches;
		}
		if (want_max && n_steps > 0) {
			DGPU_CUDA(c, cudaGraphLaunch(c->rk_graph_max, c->stream));
			c->launches += 3 * c->stage_launches;
		}
	}
	if (n_steps > 0)
		c->coef_valid = false;   // the current state is ug
	st = check_positivity_flag(c);
	if (st != DGPU_OK)
		return st;
	return read_max(c, max_rhs);
}

dgpu_status dgpu_ssp_rk3_step(dgpu_ctx* c, double dt, double* max_rhs)
{
	return dgpu_ssp_rk3_steps(c, dt, 1, max_rhs);
}

// One SSP-RK3 step from GLL coefficients `in` (device-readable) to ug and u, the new coefficients also into `out`
// (a device view of the caller's pinned buffer, or null): the first volume term keeps the coefficients (keep,
// null when they are already in u) and forms ug; the last lift writes V^-1 of the new state.
static dgpu_status enqueue_rk_step_host(dgpu_ctx* c, double dt, bool want_max, const double* in, double* keep,
                                        double* out)
{
	DGPU_CUDA(c, c->launch_volume_in(c, in, keep));
	DGPU_CUDA(c, c->launch_face(c));
	DGPU_CUDA(c, c->launch_lift_rk(c, dt, 0, 0));
	DGPU_CUDA(c, c->launch_volume_gl(c));
	DGPU_CUDA(c, c->launch_face(c));
	DGPU_CUDA(c, c->launch_lift_rk(c, dt, 1, 0));
	DGPU_CUDA(c, c->launch_volume_gl(c));
	DGPU_CUDA(c, c->launch_face(c));
	DGPU_CUDA(c, c->launch_lift_out(c, dt, want_max ? 1 : 0, out));
	return DGPU_OK;
}

dgpu_status dgpu_ssp_rk3_step_host(dgpu_ctx* c, double dt, const double* sol_in, double* sol_out, double* max_rhs)
{
	DGPU_WHOLE_MESH(c);
	if (!c || !sol_in || !sol_out || !(dt == dt))
		return DGPU_ERR_INVALID_ARGUMENT;
	if (!c->launch_volume_in || !c->launch_lift_out || c->timing) {   // Navier-Stokes, or per-kernel timing
		dgpu_status st = dgpu_upload_state(c, sol_in);
		if (st == DGPU_OK)
			st = dgpu_ssp_rk3_step(c, dt, max_rhs);
		if (st == DGPU_OK)
			st = dgpu_download_state(c, sol_out);
		return st;
	}
	const size_t bytes = state_size(c) * sizeof(double);
	const double* in = pinned_device_view(sol_in);
	double* keep = c->u;
	if (!in) {   // pageable: copy to u first
		DGPU_CUDA(c, cudaMemcpyAsync(c->u, sol_in, bytes, cudaMemcpyHostToDevice, c->stream));
		in = c->u;
		keep = nullptr;
	}
	double* out = pinned_device_view(sol_out);
	const bool want_max = (max_rhs != nullptr);
	if (!(c->host_graph && c->host_graph_dt == dt && c->host_graph_in == in && c->host_graph_out == out &&
	      c->host_graph_max == want_max)) {
		if (c->host_graph) {
			cudaGraphExecDestroy(c->host_graph);
			c->host_graph = nullptr;
		}
		cudaGraph_t g;
		DGPU_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
		const long long before = c->launches;
		dgpu_status st = enqueue_rk_step_host(c, dt, want_max, in, keep, out);
		c->launches = before;   // captured, not launched
		cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
		if (st != DGPU_OK)
			return st;
		DGPU_CUDA(c, ec);
		cudaError_t ei = cudaGraphInstantiate(&c->host_graph, g, 0);
		cudaGraphDestroy(g);
		DGPU_CUDA(c, ei);
		c->host_graph_dt = dt;
		c->host_graph_in = in;
		c->host_graph_out = out;
		c->host_graph_max = want_max;
	}
	DGPU_CUDA(c, cudaGraphLaunch(c->host_graph, c->stream));
	c->launches += 9;
	c->coef_valid = true;
	c->gl_valid = true;
	if (!out)
		DGPU_CUDA(c, cudaMemcpyAsync(sol_out, c->u, bytes, cudaMemcpyDeviceToHost, c->stream));
	dgpu_status st = check_positivity_flag(c);
	if (st != DGPU_OK)
		return st;
	st = read_max(c, max_rhs);
	if (st != DGPU_OK)
		return st;
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}

dgpu_status dgpu_positivity_corrections(dgpu_ctx* c, long long* n)
{
	if (!c || !n)
		return DGPU_ERR_INVALID_ARGUMENT;
	unsigned long long v = 0;
	DGPU_CUDA(c, cudaMemcpyAsync(&v, c->n_corr, sizeof v, cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	*n = (long long)v;
	return DGPU_OK;
}

dgpu_status dgpu_kernel_launches(const dgpu_ctx* c, long long* n)
{
	if (!c || !n)
		return DGPU_ERR_INVALID_ARGUMENT;
	*n = c->launches;
	return DGPU_OK;
}

dgpu_status dgpu_synchronize(dgpu_ctx* c)
{
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}

dgpu_status dgpu_set_stream(dgpu_ctx* c, void* stream)
{
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	if (c->own_stream)
		cudaStreamDestroy(c->stream);
	c->own_stream = false;
	c->stream = (cudaStream_t)stream;
	discard_graphs(c);
	return DGPU_OK;
}

dgpu_status dgpu_set_kernel_timing(dgpu_ctx* c, int enable)
{
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	for (auto& t : c->timers) {
		cudaEventDestroy(t.start);
		cudaEventDestroy(t.stop);
	}
	c->timers.clear();
	c->timing = enable != 0;
	return DGPU_OK;
}

dgpu_status dgpu_kernel_time(dgpu_ctx* c, const char* name, double* total_ms, long long* count)
{
	if (!c || !name || !total_ms || !count)
		return DGPU_ERR_INVALID_ARGUMENT;
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	double tot = 0.0;
	long long n = 0;
	for (auto& t : c->timers) {
		if (strcmp(t.name, name) != 0)
			continue;
		float ms = 0.f;
		DGPU_CUDA(c, cudaEventElapsedTime(&ms, t.start, t.stop));
		tot += ms;
		++n;
	}
	*total_ms = tot;
	*count = n;
	return DGPU_OK;
}

}  // extern "C"

namespace {

// FP64 FMA throughput probe: 8 independent dependency chains per thread, no memory traffic in the loop.
__global__ void fp64_fma_probe_kernel(double* out, int iters, double a, double b)
{
	double x[8];
#pragma unroll
	for (int k = 0; k < 8; ++k)
		x[k] = (threadIdx.x + 1) * 1e-9 + k;
	for (int i = 0; i < iters; ++i) {
#pragma unroll
		for (int k = 0; k < 8; ++k)
			x[k] = fma(x[k], a, b);
	}
	double s = 0.0;
#pragma unroll
	for (int k = 0; k < 8; ++k)
		s += x[k];
	out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 tensor-core throughput probe: 8 independent m8n8k4 accumulators per warp (2 * 8 * 8 * 4 flops each).
__global__ void fp64_mma_probe_kernel(double* out, int iters, double a, double b)
{
	const double av = a * (threadIdx.x + 1), bv = b;
	double d[8][2];
#pragma unroll
	for (int k = 0; k < 8; ++k) {
		d[k][0] = k;
		d[k][1] = -k;
	}
	for (int i = 0; i < iters; ++i) {
#pragma unroll
		for (int k = 0; k < 8; ++k)
			asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
			             : "+d"(d[k][0]), "+d"(d[k][1])
			             : "d"(av), "d"(bv));
	}
	double s = 0.0;
#pragma unroll
	for (int k = 0; k < 8; ++k)
		s += d[k][0] + d[k][1];
	out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

dgpu_status probe_fp64_rate(int iters, double* tflops, bool mma)
{
	if (iters < 1 || !tflops)
		return DGPU_ERR_INVALID_ARGUMENT;
	int dev = 0, sms = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
		return DGPU_ERR_NO_DEVICE;
	const int threads = 256, blocks = sms * 8;
	double* out = nullptr;
	if (cudaMalloc((void**)&out, (size_t)threads * blocks * sizeof(double)) != cudaSuccess)
		return DGPU_ERR_CUDA;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	auto* kern = mma ? fp64_mma_probe_kernel : fp64_fma_probe_kernel;
	kern<<<blocks, threads>>>(out, 16, mma ? 1e-9 : 0.999999, mma ? 0.5 : 1e-7);  // warm-up
	cudaEventRecord(e0);
	kern<<<blocks, threads>>>(out, iters, mma ? 1e-9 : 0.999999, mma ? 0.5 : 1e-7);
	cudaEventRecord(e1);
	cudaError_t e = cudaEventSynchronize(e1);
	float ms = 0.f;
	cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(out);
	if (e != cudaSuccess)
		return DGPU_ERR_CUDA;
	// per thread and iteration: 8 FMAs (FMA probe) or 8 / 32 of a warp's 8 m8n8k4 products of 512 flops
	const double flops = (mma ? 8.0 * 512.0 / 32.0 : 2.0 * 8.0) * (double)iters * threads * blocks;
	*tflops = flops / (ms * 1e-3) / 1e12;
	return DGPU_OK;
}

}  // namespace

extern "C" dgpu_status dgpu_probe_fp64(int iters, double* tflops) { return probe_fp64_rate(iters, tflops, false); }

extern "C" dgpu_status dgpu_probe_fp64_mma(int iters, double* tflops) { return probe_fp64_rate(iters, tflops, true); }

// ---------------------------------------------------------------------------------------------------------------
// Residual evaluation without any device allocation (dgpu_compute_rhs_noalloc).
//
// Some callers cannot call cudaMalloc at all: a host application whose device memory is owned by its own pool
// or framework and that hands the library only its buffers, or code that must not allocate while it runs (a
// pre-allocated real-time loop). For them the residual's intermediates -- packed geometry, connectivity, volume
// term, face traces and face fluxes -- live in one file-scope device array of fixed size instead of buffers
// owned by a dgpu_ctx. Every GPU that loads this library keeps that array until the process exits.
// ---------------------------------------------------------------------------------------------------------------

#define DGPU_NOALLOC_SCRATCH_DOUBLES ((size_t)DGPU_NOALLOC_SCRATCH_BYTES / sizeof(double))

static __device__ __align__(256) double g_noalloc_scratch[DGPU_NOALLOC_SCRATCH_DOUBLES];

namespace {

constexpr int kMaxDevices = 64;
double* g_noalloc_ptr[kMaxDevices];   // device address of g_noalloc_scratch, per device, set at first use

struct NoallocWeights {
	double w[kQMax * kQMax * kQMax];     // volume cubature weights, TP order
	double wf[kQMax * kQMax];            // face cubature weights
};

// Packs the caller's reference-layout volume data into the library's layout inside the scratch array.
template <int D, int Q>
__global__ void noalloc_pack_volumes(const NoallocWeights W, int n_vol, const double* __restrict__ metrics,
                                     const double* __restrict__ jac, double* gmet, double* inv_wJ, int* err)
{
	constexpr int N = TPShape<D, Q>::N;
	const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= (long long)n_vol * N)
		return;
	const long long v = gid / N;
	const int n = (int)(gid % N);
	const double* m = metrics + v * N * D * D;
	for (int j = 0; j < D; ++j)
		for (int i = 0; i < D; ++i)
			gmet[((v * D + j) * D + i) * N + n] = W.w[n] * m[n + (size_t)N * (i + D * j)];
	const double J = jac[v * N + n];
	if (!(J > 0.0))
		atomicExch(err, 1);
	inv_wJ[v * N + n] = 1.0 / (W.w[n] * J);
}

// Face data, connectivity (vol_face) and the inverse right-trace permutation, with bounds checks: an entry
// outside the mesh, or a (volume, local face) claimed by two face sides, raises the error flag and is skipped.
template <int D, int Q>
__global__ void noalloc_pack_faces(const NoallocWeights W, int n_vol, int n_face, const int* __restrict__ face_vol,
                                   const int* __restrict__ face_lf, const int* __restrict__ nc,
                                   const double* __restrict__ normals, const double* __restrict__ jf,
                                   double* fgeo, int* vol_face, int* nc_inv, int* err)
{
	constexpr int NF = TPShape<D, Q>::NF;
	const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= (long long)n_face * NF)
		return;
	const long long f = gid / NF;
	const int i = (int)(gid % NF);
	for (int k = 0; k < D; ++k)
		fgeo[(f * (D + 1) + k) * NF + i] = normals[(f * NF + i) * D + k];
	fgeo[(f * (D + 1) + D) * NF + i] = W.wf[i] * jf[f * NF + i];
	if (i == 0) {
		for (int s = 0; s < 2; ++s) {
			const int v = face_vol[2 * f + s], lf = face_lf[2 * f + s];
			if (v < 0 || v >= n_vol || lf < 0 || lf >= 2 * D) {
				atomicExch(err, 1);
				continue;
			}
			// each (volume, local face) belongs to exactly one face side: a second claim is a bad mesh
			if (atomicCAS(&vol_face[(size_t)v * 2 * D + lf], -1, (int)(2 * f + s)) != -1)
				atomicExch(err, 1);
		}
	}
	if (nc) {
		const int t = nc[f * NF + i];
		if (t < 0 || t >= NF)
			atomicExch(err, 1);
		else
			nc_inv[f * NF + t] = i;
	}
}

// Every (volume, local face) must have been written exactly by the face list; -1 left over means a gap.
__global__ void noalloc_check_ints(const int* a, long long n, int hi, int* err)
{
	const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (gid < n && (a[gid] < 0 || a[gid] >= hi))
		atomicExch(err, 1);
}

template <int D, int Q>
cudaError_t noalloc_pack(const NoallocWeights& W, const dgpu_mesh* m, double* gmet, double* inv_wJ, double* fgeo,
                         int* vol_face, int* nc_inv, int* err, cudaStream_t st)
{
	constexpr int N = TPShape<D, Q>::N, NF = TPShape<D, Q>::NF;
	const long long nv = (long long)m->n_volumes * N, nf = (long long)m->n_faces * NF;
	noalloc_pack_volumes<D, Q><<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(W, m->n_volumes, m->metrics_vc,
	                                                                          m->jacobian_det_vc, gmet, inv_wJ, err);
	noalloc_pack_faces<D, Q><<<(unsigned)((nf + 255) / 256), 256, 0, st>>>(
		W, m->n_volumes, m->n_faces, m->face_vol, m->face_lf, m->nc_fc, m->normals_fc, m->jacobian_det_fc, fgeo,
		vol_face, nc_inv, err);
	const long long nvf = (long long)m->n_volumes * 2 * D;
	noalloc_check_ints<<<(unsigned)((nvf + 255) / 256), 256, 0, st>>>(vol_face, nvf, 2 * m->n_faces, err);
	if (m->nc_fc)
		noalloc_check_ints<<<(unsigned)((nf + 255) / 256), 256, 0, st>>>(nc_inv, nf, NF, err);
	return cudaGetLastError();
}

template <int D>
cudaError_t noalloc_pack_q(int q, const NoallocWeights& W, const dgpu_mesh* m, double* gmet, double* inv_wJ,
                           double* fgeo, int* vol_face, int* nc_inv, int* err, cudaStream_t st)
{
	switch (q) {
	case 2: return noalloc_pack<D, 2>(W, m, gmet, inv_wJ, fgeo, vol_face, nc_inv, err, st);
	case 3: return noalloc_pack<D, 3>(W, m, gmet, inv_wJ, fgeo, vol_face, nc_inv, err, st);
	case 4: return noalloc_pack<D, 4>(W, m, gmet, inv_wJ, fgeo, vol_face, nc_inv, err, st);
	case 5: return noalloc_pack<D, 5>(W, m, gmet, inv_wJ, fgeo, vol_face, nc_inv, err, st);
	default: return cudaErrorInvalidValue;
	}
}

size_t round_up_256(size_t doubles) { return (doubles + 31) / 32 * 32; }

// Device memory of device `dev` (managed memory of any device is reachable from every device).
bool is_device_pointer(const void* p, int dev)
{
	if (!p)
		return false;
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev);
}

// Per device: 0 = not checked yet, 1 = compute capability 10.3, -1 = another device. Read once per device with
// cudaDeviceGetAttribute (cudaGetDeviceProperties fills the whole property struct, far slower).
signed char g_noalloc_cc[kMaxDevices];

}  // namespace

extern "C" dgpu_status dgpu_compute_rhs_noalloc(const dgpu_physics* phys, const dgpu_tp_operators* ops,
                                                const dgpu_mesh* d_mesh, const double* d_sol, double* d_rhs,
                                                double* max_rhs, void* cuda_stream)
{
	g_create_error.clear();
	if (!phys || !ops || !d_mesh || !d_sol || !d_rhs)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "NULL argument");
	const int d = phys->d;
	if (d != 2 && d != 3)
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "d must be 2 or 3");
	if ((d == 2 && ops->elem_type != DGPU_QUAD) || (d == 3 && ops->elem_type != DGPU_HEX))
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "element type must be QUAD (d=2) or HEX (d=3)");
	if (ops->p < 1 || ops->p > kQMax - 1)
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "p must be in 1..4");
	if (phys->pde == DGPU_PDE_ADVECTION) {
		if (phys->num_flux != DGPU_NUM_FLUX_UPWIND)
			return fail(nullptr, DGPU_ERR_UNSUPPORTED, "advection supports the upwind flux");
	} else if (phys->pde == DGPU_PDE_EULER) {
		if (phys->num_flux != DGPU_NUM_FLUX_ROE_PIKE && phys->num_flux != DGPU_NUM_FLUX_LAX_FRIEDRICHS)
			return fail(nullptr, DGPU_ERR_UNSUPPORTED, "Euler supports Roe-Pike and Lax-Friedrichs");
	} else {
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "pde must be advection or Euler");
	}
	if (!ops->cv0_vs_vc || !ops->cv1_vs_vc || !ops->cv0_vs_fc || !ops->w_vc)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "NULL operator");
	if (d_mesh->n_volumes < 1 || d_mesh->n_faces < 1)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "empty mesh");
	if (d_mesh->bc_fc || d_mesh->bc_state_fc || d_mesh->bc_data)
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "boundary faces are not supported here (use dgpu_create)");
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
		return fail(nullptr, DGPU_ERR_NO_DEVICE, "no current CUDA device");
	if (!is_device_pointer(d_sol, dev) || !is_device_pointer(d_rhs, dev) ||
	    !is_device_pointer(d_mesh->metrics_vc, dev) || !is_device_pointer(d_mesh->jacobian_det_vc, dev) ||
	    !is_device_pointer(d_mesh->face_vol, dev) || !is_device_pointer(d_mesh->face_lf, dev) ||
	    !is_device_pointer(d_mesh->normals_fc, dev) || !is_device_pointer(d_mesh->jacobian_det_fc, dev) ||
	    (d_mesh->nc_fc && !is_device_pointer(d_mesh->nc_fc, dev)))
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT,
		            "state, residual and mesh arrays must be device memory of the current device");

	const int q = ops->p + 1;
	const int N = (d == 2 ? q * q : q * q * q), NF = (d == 2 ? q : q * q);
	const int nv = (phys->pde == DGPU_PDE_EULER ? d + 2 : 1);
	const size_t n_vol = (size_t)d_mesh->n_volumes, n_face = (size_t)d_mesh->n_faces;

	// scratch layout (each region 256-byte aligned), checked against the fixed size
	const size_t o_gmet = 0;
	const size_t o_inv = o_gmet + round_up_256(n_vol * d * d * N);
	const size_t o_fgeo = o_inv + round_up_256(n_vol * N);
	const size_t o_vgl = o_fgeo + round_up_256(n_face * (d + 1) * NF);
	const size_t o_tr = o_vgl + round_up_256(n_vol * nv * N);
	const size_t o_nnf = o_tr + round_up_256(n_face * 2 * nv * NF);
	const size_t o_vf = o_nnf + round_up_256(n_face * nv * NF);
	const size_t o_nci = o_vf + round_up_256((n_vol * 2 * d + 1) / 2);
	const size_t o_misc = o_nci + round_up_256(d_mesh->nc_fc ? (n_face * NF + 1) / 2 : 0);
	const size_t total = o_misc + 32;
	if (total > DGPU_NOALLOC_SCRATCH_DOUBLES) {
		char msg[256];
		snprintf(msg, sizeof msg, "mesh needs %zu bytes of scratch; dgpu_compute_rhs_noalloc has %zu (use dgpu_create)",
		         total * sizeof(double), (size_t)DGPU_NOALLOC_SCRATCH_BYTES);
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, msg);
	}

	// set-up once per device, with that device current: its compute capability and the device address of the
	// scratch array
	if (!g_noalloc_cc[dev]) {
		int major = 0, minor = 0;
		if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
		    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess)
			return fail(nullptr, DGPU_ERR_NO_DEVICE, "cannot read the device's compute capability");
		g_noalloc_cc[dev] = (major * 10 + minor == 103) ? 1 : -1;
	}
	if (g_noalloc_cc[dev] != 1)
		return fail(nullptr, DGPU_ERR_NO_DEVICE, "device is not compute capability 10.3 (sm_103a build)");
	if (!g_noalloc_ptr[dev]) {
		double* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
		if (e != cudaSuccess || !p)
			return cuda_fail(nullptr, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
		g_noalloc_ptr[dev] = p;
	}
	double* S = g_noalloc_ptr[dev];
	cudaStream_t st = (cudaStream_t)cuda_stream;

	// host-side operator derivation (same algebra as dgpu_create)
	dgpu_ctx c;   // stack context: no device memory of its own, only views into the scratch and caller buffers
	c.d = d;
	c.q = q;
	c.N = N;
	c.NF = NF;
	c.nv = nv;
	c.pde = phys->pde;
	c.flux = phys->num_flux;
	c.positivity = 0;
	c.n_vol = d_mesh->n_volumes;
	c.n_face = d_mesh->n_faces;
	for (int k = 0; k < 3; ++k)
		c.b_adv[k] = phys->b_adv[k];
	memset(&c.ops, 0, sizeof c.ops);
	double Bm[kQMax * kQMax], Bi[kQMax * kQMax];
	for (int i = 0; i < q * q; ++i)
		Bm[i] = ops->cv0_vs_vc[i];
	if (!host_invert_small(q, Bm, Bi))
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "cv0_vs_vc is singular");
	for (int a = 0; a < q; ++a)
		for (int m = 0; m < q; ++m) {
			c.ops.B[a][m] = Bm[a * q + m];
			c.ops.Binv[a][m] = Bi[a * q + m];
			double s = 0.0;
			for (int k = 0; k < q; ++k)
				s += ops->cv1_vs_vc[a * q + k] * Bi[k * q + m];
			c.ops.Dgl[a][m] = s;
		}
	for (int s = 0; s < 2; ++s)
		for (int m = 0; m < q; ++m) {
			double acc = 0.0;
			for (int k = 0; k < q; ++k)
				acc += ops->cv0_vs_fc[s * q + k] * Bi[k * q + m];
			c.ops.lb[s][m] = acc;
		}
	NoallocWeights W;
	memset(&W, 0, sizeof W);
	for (int n = 0; n < N; ++n) {
		int r = n;
		double x = 1.0;
		for (int k = 0; k < d; ++k) {
			x *= ops->w_vc[r % q];
			r /= q;
		}
		W.w[n] = x;
	}
	for (int n = 0; n < NF; ++n) {
		int r = n;
		double x = 1.0;
		for (int k = 0; k < d - 1; ++k) {
			x *= ops->w_vc[r % q];
			r /= q;
		}
		W.wf[n] = x;
	}

	int* vol_face = reinterpret_cast<int*>(S + o_vf);
	int* nc_inv = d_mesh->nc_fc ? reinterpret_cast<int*>(S + o_nci) : nullptr;
	unsigned long long* max_bits = reinterpret_cast<unsigned long long*>(S + o_misc);
	int* err = reinterpret_cast<int*>(S + o_misc + 1);
	c.u = const_cast<double*>(d_sol);
	c.rhs = d_rhs;
	c.gmet = S + o_gmet;
	c.inv_wJ = S + o_inv;
	c.fgeo = S + o_fgeo;
	c.vol_gl = S + o_vgl;
	c.traces = S + o_tr;
	c.nnf = S + o_nnf;
	c.vol_face = vol_face;
	c.nc = const_cast<int*>(d_mesh->nc_fc);
	c.nc_inv = nc_inv;
	c.max_bits = max_bits;
	c.err_flag = err;
	c.n_corr = nullptr;
	c.stream = st;
	c.own_stream = false;

	// the previous call's contents are still in the array: reset what must start cleared
	DGPU_CUDA(nullptr, cudaMemsetAsync(vol_face, 0xff, n_vol * 2 * d * sizeof(int), st));
	if (nc_inv)
		DGPU_CUDA(nullptr, cudaMemsetAsync(nc_inv, 0xff, n_face * NF * sizeof(int), st));
	DGPU_CUDA(nullptr, cudaMemsetAsync(err, 0, sizeof(int), st));
	cudaError_t pe = (d == 2 ? noalloc_pack_q<2>(q, W, d_mesh, c.gmet, c.inv_wJ, c.fgeo, vol_face, nc_inv, err, st)
	                         : noalloc_pack_q<3>(q, W, d_mesh, c.gmet, c.inv_wJ, c.fgeo, vol_face, nc_inv, err, st));
	DGPU_CUDA(nullptr, pe);
	int h_err = 0;
	DGPU_CUDA(nullptr, cudaMemcpyAsync(&h_err, err, sizeof h_err, cudaMemcpyDeviceToHost, st));
	DGPU_CUDA(nullptr, cudaStreamSynchronize(st));
	if (h_err)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT,
		            "bad mesh: a face index, local face, permutation or jacobian_det_vc is out of range");

	// the residual kernels of dgpu_compute_rhs, unchanged, on the scratch views
	DGPU_CUDA(nullptr, d == 2 ? bind_q<2>(&c) : bind_q<3>(&c));
	DGPU_CUDA(nullptr, c.launch_volume(&c));
	DGPU_CUDA(nullptr, c.launch_face(&c));
	DGPU_CUDA(nullptr, c.launch_lift_rhs(&c));
	if (max_rhs) {
		unsigned long long bits = 0;
		DGPU_CUDA(nullptr, cudaMemcpyAsync(&bits, max_bits, sizeof bits, cudaMemcpyDeviceToHost, st));
		DGPU_CUDA(nullptr, cudaStreamSynchronize(st));
		double v;
		memcpy(&v, &bits, sizeof v);
		*max_rhs = v;
	}
	return DGPU_OK;
}

// ---------------------------------------------------------------------------------------------------------------
// Discrete adjoint: forward/backward pair shaped like an autograd Function.
// ---------------------------------------------------------------------------------------------------------------
namespace {

dgpu_status ensure_adjoint_buffers(dgpu_ctx* c)
{
	if (c->u_saved)
		return DGPU_OK;
	const size_t ns = state_size(c);
	const size_t nt = (size_t)c->n_face * 2 * c->nv * c->NF;
	DGPU_CUDA(c, cudaMalloc((void**)&c->u_saved, ns * sizeof(double)));
	DGPU_CUDA(c, cudaMalloc((void**)&c->vbar, ns * sizeof(double)));
	DGPU_CUDA(c, cudaMalloc((void**)&c->ubar, ns * sizeof(double)));
	DGPU_CUDA(c, cudaMalloc((void**)&c->atraces, nt * sizeof(double)));
	DGPU_CUDA(c, cudaMalloc((void**)&c->wbar, nt * sizeof(double)));
	if (c->ns) {
		DGPU_CUDA(c, cudaMalloc((void**)&c->ns_gbar, ns * c->d * sizeof(double)));
		DGPU_CUDA(c, cudaMalloc((void**)&c->ns_xbar, nt * c->d * sizeof(double)));
		DGPU_CUDA(c, cudaMalloc((void**)&c->ns_gtbar, nt * c->d * sizeof(double)));
	}
	return DGPU_OK;
}

}  // namespace

namespace {

dgpu_status ensure_jvp_buffers(dgpu_ctx* c)
{
	const size_t ns = state_size(c);
	const size_t nt = (size_t)c->n_face * 2 * c->nv * c->NF;
	if (!c->jv_du) {
		DGPU_CUDA(c, cudaMalloc((void**)&c->jv_du, ns * sizeof(double)));
		DGPU_CUDA(c, cudaMalloc((void**)&c->jv_vol, ns * sizeof(double)));
		DGPU_CUDA(c, cudaMalloc((void**)&c->jv_out, ns * sizeof(double)));
		DGPU_CUDA(c, cudaMalloc((void**)&c->jv_traces, nt * sizeof(double)));
		DGPU_CUDA(c, cudaMalloc((void**)&c->jv_nnf, nt / 2 * sizeof(double)));
	}
	if (c->ns && !c->ns_gv_d) {
		DGPU_CUDA(c, cudaMalloc((void**)&c->ns_gtr_d, nt * c->d * sizeof(double)));
		DGPU_CUDA(c, cudaMalloc((void**)&c->ns_X_d, nt / 2 * c->d * sizeof(double)));
		DGPU_CUDA(c, cudaMalloc((void**)&c->ns_gv_d, ns * c->d * sizeof(double)));
	}
	return DGPU_OK;
}

// Block rows (volume v: itself and its face neighbours, ascending, each once), a greedy distance-2 colouring (no
// block row holds two volumes of one colour) and, per (volume, colour), the slot of the block whose column volume
// has that colour (-1 when none).
dgpu_status jacobian_setup(dgpu_ctx* c)
{
	if (c->jac_colours > 0)
		return DGPU_OK;
	const int nV = c->n_vol;
	std::vector<std::vector<int>> cols(nV);
	for (int v = 0; v < nV; ++v)
		cols[v].push_back(v);
	for (int f = 0; f < c->n_face; ++f) {
		const int a = c->h_face_vol[2 * f], b = c->h_face_vol[2 * f + 1];
		if (b < 0)
			continue;   // boundary face: no coupling
		cols[a].push_back(b);
		cols[b].push_back(a);
	}
	c->jac_row_ptr.assign(nV + 1, 0);
	c->jac_col_idx.clear();
	for (int v = 0; v < nV; ++v) {
		std::sort(cols[v].begin(), cols[v].end());
		cols[v].erase(std::unique(cols[v].begin(), cols[v].end()), cols[v].end());
		c->jac_row_ptr[v + 1] = c->jac_row_ptr[v] + (int)cols[v].size();
		c->jac_col_idx.insert(c->jac_col_idx.end(), cols[v].begin(), cols[v].end());
	}
	std::vector<int> colour(nV, -1), stamp;
	int n_col = 0;
	for (int v = 0; v < nV; ++v) {
		for (int r : cols[v])          // the rows that hold v ...
			for (int y : cols[r])      // ... and every volume in them
				if (colour[y] >= 0)
					stamp[colour[y]] = v + 1;
		int k = 0;
		while (k < n_col && stamp[k] == v + 1)
			++k;
		if (k == n_col) {
			++n_col;
			stamp.push_back(0);
		}
		colour[v] = k;
	}
	std::vector<int> slot((size_t)nV * n_col, -1);
	for (int v = 0; v < nV; ++v)
		for (int j = c->jac_row_ptr[v]; j < c->jac_row_ptr[v + 1]; ++j) {
			int& s = slot[(size_t)v * n_col + colour[c->jac_col_idx[j]]];
			if (s != -1)
				return fail(c, DGPU_ERR_INVALID_ARGUMENT, "internal: colouring is not distance-2");
			s = j;
		}
	c->jac_members_off.assign(n_col + 1, 0);
	for (int v = 0; v < nV; ++v)
		++c->jac_members_off[colour[v] + 1];
	for (int k = 0; k < n_col; ++k)
		c->jac_members_off[k + 1] += c->jac_members_off[k];
	std::vector<int> members(nV), fill(c->jac_members_off.begin(), c->jac_members_off.end() - 1);
	for (int v = 0; v < nV; ++v)
		members[fill[colour[v]]++] = v;
	DGPU_CUDA(c, upload(&c->jac_slot, slot));
	DGPU_CUDA(c, upload(&c->jac_members, members));
	c->jac_colours = n_col;
	return DGPU_OK;
}

}  // namespace

extern "C" dgpu_status dgpu_jacobian_structure(dgpu_ctx* c, int* block_size, long long* n_blocks, int* n_colours)
{
	DGPU_WHOLE_MESH(c);
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	const dgpu_status st = jacobian_setup(c);
	if (st != DGPU_OK)
		return st;
	if (block_size)
		*block_size = c->nv * c->N;
	if (n_blocks)
		*n_blocks = (long long)c->jac_col_idx.size();
	if (n_colours)
		*n_colours = c->jac_colours;
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_jacobian_bsr(dgpu_ctx* c, const double* sol, int raw, int* row_ptr, int* col_idx,
                                         double* values)
{
	DGPU_WHOLE_MESH(c);
	if (!c || !sol)
		return DGPU_ERR_INVALID_ARGUMENT;
	dgpu_status st = jacobian_setup(c);
	if (st == DGPU_OK)
		st = ensure_jvp_buffers(c);
	if (st != DGPU_OK)
		return st;
	if (row_ptr)
		memcpy(row_ptr, c->jac_row_ptr.data(), c->jac_row_ptr.size() * sizeof(int));
	if (col_idx)
		memcpy(col_idx, c->jac_col_idx.data(), c->jac_col_idx.size() * sizeof(int));
	if (!values)
		return DGPU_OK;
	const int nb = c->nv * c->N, n_col = c->jac_colours;
	const size_t n_vals = c->jac_col_idx.size() * (size_t)nb * nb, ns = state_size(c);
	cudaPointerAttributes pa;
	bool dev_out = false;
	if (cudaPointerGetAttributes(&pa, values) == cudaSuccess)
		dev_out = (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged);
	else
		cudaGetLastError();
	double* vals = values;
	double* mass_out = nullptr;
	if (!dev_out) {
		cudaError_t e = cudaMalloc((void**)&vals, n_vals * sizeof(double));
		if (e != cudaSuccess)
			return fail(c, DGPU_ERR_CUDA, "dgpu_jacobian_bsr: no device memory for the staging copy of " +
			                                  std::to_string(n_vals * sizeof(double)) + " bytes of blocks");
	}
	cudaError_t e = raw ? cudaMalloc((void**)&mass_out, ns * sizeof(double)) : cudaSuccess;
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(c->u, sol, ns * sizeof(double), cudaMemcpyHostToDevice, c->stream);
	if (e == cudaSuccess)
		e = cudaMemsetAsync(c->jv_du, 0, ns * sizeof(double), c->stream);
	c->coef_valid = true;
	c->gl_valid = false;
	const long long nrows = (long long)c->n_vol * nb;
	for (int col = 0; col < n_col && e == cudaSuccess; ++col) {
		const int m0 = c->jac_members_off[col], nm = c->jac_members_off[col + 1] - m0;
		const unsigned gs = (unsigned)((nm + 255) / 256), gr = (unsigned)((nrows + 255) / 256);
		for (int k = 0; k < nb && e == cudaSuccess; ++k) {
			jac_seed_kernel<<<gs, 256, 0, c->stream>>>(c->jv_du, c->jac_members + m0, nm, nb, k, 1.0);
			e = c->launch_jvp_tangent(c);
			const double* jv = c->jv_out;
			if (e == cudaSuccess && raw) {
				e = c->launch_mass(c, c->jv_out, mass_out);
				jv = mass_out;
			}
			jac_scatter_kernel<<<gr, 256, 0, c->stream>>>(jv, c->jac_slot, n_col, col, c->n_vol, nb, k, vals);
			jac_seed_kernel<<<gs, 256, 0, c->stream>>>(c->jv_du, c->jac_members + m0, nm, nb, k, 0.0);
			c->launches += 3;
			if (e == cudaSuccess)
				e = cudaGetLastError();
		}
	}
	if (e == cudaSuccess && !dev_out)
		e = cudaMemcpyAsync(values, vals, n_vals * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(c->stream);
	if (!dev_out)
		cudaFree(vals);
	if (mass_out)
		cudaFree(mass_out);
	if (e != cudaSuccess)
		return cuda_fail(c, e, "dgpu_jacobian_bsr");
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_jvp(dgpu_ctx* c, const double* sol, const double* dir, double* rhs, double* jv)
{
	DGPU_WHOLE_MESH(c);
	if (!c || !sol || !dir || !jv)
		return DGPU_ERR_INVALID_ARGUMENT;
	const size_t ns = state_size(c);
	{
		const dgpu_status st = ensure_jvp_buffers(c);
		if (st != DGPU_OK)
			return st;
	}
	const size_t bytes = ns * sizeof(double);
	DGPU_CUDA(c, cudaMemcpyAsync(c->u, sol, bytes, cudaMemcpyHostToDevice, c->stream));
	DGPU_CUDA(c, cudaMemcpyAsync(c->jv_du, dir, bytes, cudaMemcpyHostToDevice, c->stream));
	c->coef_valid = true;
	c->gl_valid = false;
	DGPU_CUDA(c, c->launch_jvp(c));
	if (rhs)
		DGPU_CUDA(c, cudaMemcpyAsync(rhs, c->rhs, bytes, cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaMemcpyAsync(jv, c->jv_out, bytes, cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_vjp_forward(dgpu_ctx* c, const double* sol, double* rhs, double* max_rhs)
{
	DGPU_WHOLE_MESH(c);
	if (!c || !sol)
		return DGPU_ERR_INVALID_ARGUMENT;
	dgpu_status st = ensure_adjoint_buffers(c);
	if (st != DGPU_OK)
		return st;
	const size_t bytes = state_size(c) * sizeof(double);
	DGPU_CUDA(c, cudaMemcpyAsync(c->u_saved, sol, bytes, cudaMemcpyHostToDevice, c->stream));
	DGPU_CUDA(c, cudaMemcpyAsync(c->u, c->u_saved, bytes, cudaMemcpyDeviceToDevice, c->stream));
	c->coef_valid = true;
	c->gl_valid = false;
	st = enqueue_rhs(c);
	if (st != DGPU_OK)
		return st;
	if (rhs)
		DGPU_CUDA(c, cudaMemcpyAsync(rhs, c->rhs, bytes, cudaMemcpyDeviceToHost, c->stream));
	if (max_rhs)
		return read_max(c, max_rhs);
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_vjp_backward(dgpu_ctx* c, const double* cotangent, double* grad_sol)
{
	DGPU_WHOLE_MESH(c);
	if (!c || !cotangent || !grad_sol)
		return DGPU_ERR_INVALID_ARGUMENT;
	if (!c->u_saved)
		return fail(c, DGPU_ERR_INVALID_ARGUMENT, "dgpu_vjp_backward needs a preceding dgpu_vjp_forward");
	const size_t bytes = state_size(c) * sizeof(double);
	DGPU_CUDA(c, cudaMemcpyAsync(c->vbar, cotangent, bytes, cudaMemcpyHostToDevice, c->stream));
	DGPU_CUDA(c, c->launch_adjoint(c, c->u_saved, c->vbar, c->ubar));
	DGPU_CUDA(c, cudaMemcpyAsync(grad_sol, c->ubar, bytes, cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}

// ---------------------------------------------------------------------------------------------------------------
// Objective J = integral of pressure over a set of faces, and the adjoint of n SSP-RK3 steps of J.
// ---------------------------------------------------------------------------------------------------------------
extern "C" dgpu_status dgpu_set_objective_faces(dgpu_ctx* c, int n_faces, const int* faces)
{
	DGPU_WHOLE_MESH(c);
	if (!c || n_faces < 1 || !faces)
		return DGPU_ERR_INVALID_ARGUMENT;
	if (c->pde != DGPU_PDE_EULER && c->pde != DGPU_PDE_NAVIER_STOKES)
		return fail(c, DGPU_ERR_UNSUPPORTED, "the pressure objective needs the Euler or Navier-Stokes equations");
	for (int i = 0; i < n_faces; ++i)
		if (faces[i] < 0 || faces[i] >= c->n_face)
			return fail(c, DGPU_ERR_INVALID_ARGUMENT, "objective face index out of range");
	dgpu_status st = ensure_adjoint_buffers(c);
	if (st != DGPU_OK)
		return st;
	if (c->obj_faces) {
		cudaFree(c->obj_faces);
		cudaFree(c->obj_contrib);
		c->obj_faces = nullptr;
		c->obj_contrib = nullptr;
	}
	DGPU_CUDA(c, cudaMalloc((void**)&c->obj_faces, n_faces * sizeof(int)));
	DGPU_CUDA(c, cudaMalloc((void**)&c->obj_contrib, (size_t)n_faces * c->NF * sizeof(double)));
	DGPU_CUDA(c, cudaMemcpy(c->obj_faces, faces, n_faces * sizeof(int), cudaMemcpyHostToDevice));
	c->n_obj = n_faces;
	return DGPU_OK;
}

namespace {

// J at the device state d_u (GLL), summed on the host in face-node order (deterministic); dJ/du into d_grad
// when not null. Uses the forward volume kernel for the traces (its volume term output is overwritten).
dgpu_status objective_at(dgpu_ctx* c, double* d_u, double* J, double* d_grad)
{
	double* keep = c->u;
	c->u = d_u;
	cudaError_t e = c->launch_volume(c);
	c->u = keep;
	DGPU_CUDA(c, e);
	DGPU_CUDA(c, c->launch_objective(c, d_grad));
	std::vector<double> h((size_t)c->n_obj * c->NF);
	DGPU_CUDA(c, cudaMemcpyAsync(h.data(), c->obj_contrib, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
	                             c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	double s = 0.0;
	for (double x : h)
		s += x;
	*J = s;
	return DGPU_OK;
}

dgpu_status lincomb(dgpu_ctx* c, double a, const double* x, double b, const double* y, double cc, const double* z,
                    double* out)
{
	const size_t n = state_size(c);
	lincomb_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, a, x, b, y, cc, z, out);
	c->launches++;
	DGPU_CUDA(c, cudaGetLastError());
	return DGPU_OK;
}

// R(x) into c->rhs (the residual kernels read the state from c->u).
dgpu_status residual_of(dgpu_ctx* c, double* x)
{
	double* keep = c->u;
	c->u = x;
	dgpu_status st = enqueue_rhs(c);
	c->u = keep;
	return st;
}

// One SSP-RK3 step on GLL coefficients (the expressions of solve_explicit.c:277-295, without the positivity
// limiter, whose corrections are not differentiable): x -> y; s1, s2 receive the stage states.
dgpu_status rk3_gll_step(dgpu_ctx* c, double dt, double* x, double* s1, double* s2, double* y)
{
	dgpu_status st;
	if ((st = residual_of(c, x)) != DGPU_OK) return st;
	if ((st = lincomb(c, 1.0, x, dt, c->rhs, 0.0, nullptr, s1)) != DGPU_OK) return st;
	if ((st = residual_of(c, s1)) != DGPU_OK) return st;
	if ((st = lincomb(c, 0.75, x, 0.25, s1, 0.25 * dt, c->rhs, s2)) != DGPU_OK) return st;
	if ((st = residual_of(c, s2)) != DGPU_OK) return st;
	return lincomb(c, 1.0 / 3.0, x, 2.0 / 3.0, s2, 2.0 / 3.0 * dt, c->rhs, y);
}

struct DeviceBlock {
	double* p = nullptr;
	~DeviceBlock() { if (p) cudaFree(p); }
};

}  // namespace

extern "C" dgpu_status dgpu_objective(dgpu_ctx* c, const double* sol, double* J, double* dJ_dsol)
{
	DGPU_WHOLE_MESH(c);
	if (!c || !sol || !J)
		return DGPU_ERR_INVALID_ARGUMENT;
	if (!c->obj_faces)
		return fail(c, DGPU_ERR_INVALID_ARGUMENT, "no objective faces: call dgpu_set_objective_faces");
	const size_t bytes = state_size(c) * sizeof(double);
	DGPU_CUDA(c, cudaMemcpyAsync(c->vbar, sol, bytes, cudaMemcpyHostToDevice, c->stream));
	dgpu_status st = objective_at(c, c->vbar, J, dJ_dsol ? c->ubar : nullptr);
	if (st != DGPU_OK || !dJ_dsol)
		return st;
	DGPU_CUDA(c, cudaMemcpyAsync(dJ_dsol, c->ubar, bytes, cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_adjoint_ssp_rk3(dgpu_ctx* c, double dt, int n_steps, size_t budget_bytes,
                                            const double* sol0, double* J, double* dJ_dsol0, int* segment_out)
{
	DGPU_WHOLE_MESH(c);
	if (!c || n_steps < 1 || !sol0 || !J || !dJ_dsol0 || !(dt == dt))
		return DGPU_ERR_INVALID_ARGUMENT;
	if (!c->obj_faces)
		return fail(c, DGPU_ERR_INVALID_ARGUMENT, "no objective faces: call dgpu_set_objective_faces");
	const size_t ns = state_size(c), sb = ns * sizeof(double);
	// K states per recomputed segment, C checkpoints, 7 work vectors: (C + K + 7) states within the budget
	int best_k = -1;
	size_t best_total = 0;
	for (int K = 1; K <= n_steps; ++K) {
		const int C = (n_steps + K - 1) / K;
		const size_t total = (size_t)(C + K + 7) * sb;
		if (total <= budget_bytes && (best_k < 0 || total < best_total)) {
			best_k = K;
			best_total = total;
		}
	}
	if (best_k < 0) {
		char msg[160];
		snprintf(msg, sizeof msg, "adjoint of %d steps needs at least %zu bytes of device memory", n_steps,
		         (size_t)(2 * (size_t)ceil(sqrt((double)n_steps)) + 7) * sb);
		return fail(c, DGPU_ERR_INVALID_ARGUMENT, msg);
	}
	const int K = best_k, C = (n_steps + K - 1) / K;
	DeviceBlock blk;
	DGPU_CUDA(c, cudaMalloc((void**)&blk.p, best_total));
	double* chk = blk.p;                           // C checkpoints: states at steps 0, K, 2K, ...
	double* seg = chk + (size_t)C * ns;            // K states of the segment being reversed
	double* s1 = seg + (size_t)K * ns;
	double* s2 = s1 + ns;
	double* ub = s2 + ns;                          // cotangent of the current state
	double* sb0 = ub + ns;
	double* sb2 = sb0 + ns;
	double* rb = sb2 + ns;
	double* g = rb + ns;
	DGPU_CUDA(c, cudaMemcpyAsync(chk, sol0, sb, cudaMemcpyHostToDevice, c->stream));
	dgpu_status st;
	// forward sweep, keeping every K-th state
	double* cur = chk;
	double* tmp[2] = {ub, g};   // ping-pong for the states between checkpoints
	int t = 0;
	for (int n = 0; n < n_steps; ++n) {
		double* nxt;
		if ((n + 1) % K == 0 && (n + 1) / K < C) {
			nxt = chk + (size_t)((n + 1) / K) * ns;
		} else {
			nxt = tmp[t];
			t ^= 1;
		}
		if ((st = rk3_gll_step(c, dt, cur, s1, s2, nxt)) != DGPU_OK)
			return st;
		cur = nxt;
	}
	if ((st = objective_at(c, cur, J, ub)) != DGPU_OK)
		return st;
	// backward sweep, segment by segment
	for (int sgi = C - 1; sgi >= 0; --sgi) {
		const int n0 = sgi * K, n1 = (n0 + K < n_steps) ? n0 + K : n_steps;
		DGPU_CUDA(c, cudaMemcpyAsync(seg, chk + (size_t)sgi * ns, sb, cudaMemcpyDeviceToDevice, c->stream));
		for (int n = n0 + 1; n < n1; ++n)
			if ((st = rk3_gll_step(c, dt, seg + (size_t)(n - 1 - n0) * ns, s1, s2, seg + (size_t)(n - n0) * ns)) != DGPU_OK)
				return st;
		for (int n = n1 - 1; n >= n0; --n) {
			double* s0 = seg + (size_t)(n - n0) * ns;
			// stage states of step n (recomputed, not stored)
			if ((st = residual_of(c, s0)) != DGPU_OK) return st;
			if ((st = lincomb(c, 1.0, s0, dt, c->rhs, 0.0, nullptr, s1)) != DGPU_OK) return st;
			if ((st = residual_of(c, s1)) != DGPU_OK) return st;
			if ((st = lincomb(c, 0.75, s0, 0.25, s1, 0.25 * dt, c->rhs, s2)) != DGPU_OK) return st;
			// y = 1/3 s0 + 2/3 s2 + 2/3 dt R(s2)
			if ((st = lincomb(c, 2.0 / 3.0 * dt, ub, 0.0, ub, 0.0, nullptr, rb)) != DGPU_OK) return st;
			DGPU_CUDA(c, c->launch_adjoint(c, s2, rb, g));
			if ((st = lincomb(c, 2.0 / 3.0, ub, 1.0, g, 0.0, nullptr, sb2)) != DGPU_OK) return st;
			if ((st = lincomb(c, 1.0 / 3.0, ub, 0.0, ub, 0.0, nullptr, sb0)) != DGPU_OK) return st;
			// s2 = 3/4 s0 + 1/4 s1 + 1/4 dt R(s1)
			if ((st = lincomb(c, 0.25 * dt, sb2, 0.0, sb2, 0.0, nullptr, rb)) != DGPU_OK) return st;
			DGPU_CUDA(c, c->launch_adjoint(c, s1, rb, g));
			if ((st = lincomb(c, 0.25, sb2, 1.0, g, 0.0, nullptr, s1)) != DGPU_OK) return st;      // s1 <- sbar1
			if ((st = lincomb(c, 1.0, sb0, 0.75, sb2, 0.0, nullptr, sb0)) != DGPU_OK) return st;
			// s1 = s0 + dt R(s0)
			if ((st = lincomb(c, dt, s1, 0.0, s1, 0.0, nullptr, rb)) != DGPU_OK) return st;
			DGPU_CUDA(c, c->launch_adjoint(c, s0, rb, g));
			if ((st = lincomb(c, 1.0, sb0, 1.0, s1, 1.0, g, ub)) != DGPU_OK) return st;
		}
	}
	DGPU_CUDA(c, cudaMemcpyAsync(dJ_dsol0, ub, sb, cudaMemcpyDeviceToHost, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	if (segment_out)
		*segment_out = K;
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_compute_geometry(int d, const dgpu_tp_operators* ops, const dgpu_mesh* mesh,
                                             double* metrics_vc, double* jacobian_det_vc, double* normals_fc,
                                             double* jacobian_det_fc, double* xyz_fc)
{
	g_create_error.clear();
	if (!ops || !mesh || !mesh->geom_coef || !ops->w_vc)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "NULL argument (geom_coef and w_vc are needed)");
	if ((d == 2 && ops->elem_type != DGPU_QUAD) || (d == 3 && ops->elem_type != DGPU_HEX) || (d != 2 && d != 3))
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "element type must be QUAD (d=2) or HEX (d=3)");
	if (ops->p < 1 || ops->p > kQMax - 1 || mesh->p_g < 1 || mesh->p_g > kQMax - 1)
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "p and p_g must be in 1..4");
	if (mesh->n_volumes < 1 || mesh->n_faces < 0 || (mesh->n_faces > 0 && (!mesh->face_vol || !mesh->face_lf)))
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "incomplete mesh");
	for (int f = 0; f < mesh->n_faces; ++f)
		if (mesh->face_vol[2 * f] < 0 || mesh->face_vol[2 * f] >= mesh->n_volumes || mesh->face_lf[2 * f] < 0 ||
		    mesh->face_lf[2 * f] >= 2 * d)
			return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "bad face connectivity (side 0)");
	int n_dev = 0;
	if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev < 1)
		return fail(nullptr, DGPU_ERR_NO_DEVICE, "no CUDA device");

	const int q = ops->p + 1;
	const size_t nv = (size_t)mesh->n_volumes, nf = (size_t)mesh->n_faces;
	const size_t nc = (d == 2 ? q * q : q * q * q), nfc = (d == 2 ? q : q * q);
	GeoOps G;
	build_geo_ops(d, q, mesh->p_g, ops->w_vc, &G);
	GeoBuffers B;
	struct Result {
		double* host;
		size_t n;
		double* dev;
	} res[5] = {{metrics_vc, nv * d * d * nc, nullptr}, {jacobian_det_vc, nv * nc, nullptr},
	            {normals_fc, nf * nfc * d, nullptr}, {jacobian_det_fc, nf * nfc, nullptr},
	            {xyz_fc, nf * nfc * d, nullptr}};
	cudaStream_t st = nullptr;
	cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
	for (auto& r : res)
		if (e == cudaSuccess && r.host && r.n > 0)
			e = cudaMalloc((void**)&r.dev, r.n * sizeof(double));
	if (e == cudaSuccess)
		e = B.init(mesh, d, st);
	int h_err = 0;
	if (e == cudaSuccess) {
		GeoOut out = {};
		out.metrics_vc = res[0].dev;
		out.jacobian_det_vc = res[1].dev;
		out.normals_fc = res[2].dev;
		out.jacobian_det_fc = res[3].dev;
		out.xyz_fc = res[4].dev;
		e = B.run(G, mesh, out, st, &h_err);
	}
	for (auto& r : res)
		if (e == cudaSuccess && r.dev)
			e = cudaMemcpyAsync(r.host, r.dev, r.n * sizeof(double), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(st);
	for (auto& r : res)
		if (r.dev)
			cudaFree(r.dev);
	if (st)
		cudaStreamDestroy(st);
	if (e != cudaSuccess)
		return cuda_fail(nullptr, e, "dgpu_compute_geometry");
	if (h_err)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "non-positive Jacobian determinant");
	return DGPU_OK;
}

extern "C" dgpu_status dgpu_blend_geometry(int d, int p_g, int n_volumes, const double* xyz_ve, const int* face_curved,
                                           double* geom_coef)
{
	g_create_error.clear();
	if (!xyz_ve || !face_curved || !geom_coef || n_volumes < 1)
		return fail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "NULL argument or no volumes");
	if (d != 2)
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "blended geometry is provided for QUAD volumes (d = 2) only");
	if (p_g < 1 || p_g > kQMax - 1)
		return fail(nullptr, DGPU_ERR_UNSUPPORTED, "p_g must be in 1..4");
	int n_dev = 0;
	if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev < 1)
		return fail(nullptr, DGPU_ERR_NO_DEVICE, "no CUDA device");
	BlendArgs A = {};
	A.n_vol = n_volumes;
	A.qg = p_g + 1;
	gauss_lobatto_nodes(A.qg, A.x);
	const size_t nv = (size_t)n_volumes, n_g = (size_t)A.qg * A.qg;
	cudaStream_t st = nullptr;
	double *d_ve = nullptr, *d_out = nullptr;
	int* d_fc = nullptr;
	cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
	if (e == cudaSuccess)
		e = cudaMalloc((void**)&d_ve, nv * 8 * sizeof(double));
	if (e == cudaSuccess)
		e = cudaMalloc((void**)&d_fc, nv * 4 * sizeof(int));
	if (e == cudaSuccess)
		e = cudaMalloc((void**)&d_out, nv * 2 * n_g * sizeof(double));
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(d_ve, xyz_ve, nv * 8 * sizeof(double), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(d_fc, face_curved, nv * 4 * sizeof(int), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) {
		A.xyz_ve = d_ve;
		A.face_curved = d_fc;
		A.geom_coef = d_out;
		blend_quad_kernel<<<(unsigned)((nv + 127) / 128), 128, 0, st>>>(A);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(geom_coef, d_out, nv * 2 * n_g * sizeof(double), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(st);
	cudaFree(d_ve);
	cudaFree(d_fc);
	cudaFree(d_out);
	if (st)
		cudaStreamDestroy(st);
	if (e != cudaSuccess)
		return cuda_fail(nullptr, e, "dgpu_blend_geometry");
	return DGPU_OK;
}

// ---------------------------------------------------------------------------------------------------------------
// Element partitions: the residual and the SSP-RK3 stages in two halves around the exchange of the traces of the
// faces cut by the partition (one process per GPU, the exchange by the caller, e.g. NCCL send/recv on the context's
// stream). The reference runs on one process; this is the distributed form of compute_rhs_dg / time_step_ssp_rk_33.
// ---------------------------------------------------------------------------------------------------------------
extern "C" {

dgpu_status dgpu_halo_setup(dgpu_ctx* c, int n_slots, const int* send_slots, const int* recv_slots)
{
	if (!c || n_slots < 0 || (n_slots > 0 && (!send_slots || !recv_slots)))
		return DGPU_ERR_INVALID_ARGUMENT;
	if (c->n_halo > 0 || c->halo_send)
		return fail(c, DGPU_ERR_INVALID_ARGUMENT, "the halo is already set up");
	if (n_slots != c->n_remote)
		return fail(c, DGPU_ERR_INVALID_ARGUMENT,
		            "the halo must receive every remote face side once: " + std::to_string(c->n_remote) + " sides, " +
		                std::to_string(n_slots) + " slots");
	std::vector<char> seen(2 * (size_t)c->n_face, 0);
	for (int i = 0; i < n_slots; ++i) {
		const int a = send_slots[i], b = recv_slots[i];
		if (a < 0 || b < 0 || a >= 2 * c->n_face || b >= 2 * c->n_face || a / 2 != b / 2 || a == b ||
		    c->h_face_vol[a] < 0 || c->h_face_vol[b] != DGPU_REMOTE_VOLUME || seen[b])
			return fail(c, DGPU_ERR_INVALID_ARGUMENT,
			            "halo slot " + std::to_string(i) + ": send the local side and receive the remote side of a face");
		seen[b] = 1;
	}
	if (n_slots == 0)
		return DGPU_OK;
	const size_t slot = (size_t)c->nv * c->NF;
	DGPU_CUDA(c, cudaMalloc((void**)&c->halo_send, n_slots * sizeof(int)));
	DGPU_CUDA(c, cudaMalloc((void**)&c->halo_recv, n_slots * sizeof(int)));
	DGPU_CUDA(c, cudaMalloc((void**)&c->halo_sbuf, n_slots * slot * sizeof(double)));
	DGPU_CUDA(c, cudaMalloc((void**)&c->halo_rbuf, n_slots * slot * sizeof(double)));
	DGPU_CUDA(c, cudaMemcpy(c->halo_send, send_slots, n_slots * sizeof(int), cudaMemcpyHostToDevice));
	DGPU_CUDA(c, cudaMemcpy(c->halo_recv, recv_slots, n_slots * sizeof(int), cudaMemcpyHostToDevice));
	DGPU_CUDA(c, cudaMemset(c->halo_sbuf, 0, n_slots * slot * sizeof(double)));
	DGPU_CUDA(c, cudaMemset(c->halo_rbuf, 0, n_slots * slot * sizeof(double)));
	c->n_halo = n_slots;
	return DGPU_OK;
}

dgpu_status dgpu_halo_buffers(dgpu_ctx* c, double** d_send, double** d_recv, size_t* slot_doubles)
{
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	if (d_send)
		*d_send = c->halo_sbuf;
	if (d_recv)
		*d_recv = c->halo_rbuf;
	if (slot_doubles)
		*slot_doubles = (size_t)c->nv * c->NF;
	return DGPU_OK;
}

dgpu_status dgpu_get_stream(dgpu_ctx* c, void** cuda_stream)
{
	if (!c || !cuda_stream)
		return DGPU_ERR_INVALID_ARGUMENT;
	*cuda_stream = (void*)c->stream;
	return DGPU_OK;
}

static dgpu_status halo_ready(dgpu_ctx* c)
{
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	if (c->n_remote > 0 && c->n_halo != c->n_remote)
		return fail(c, DGPU_ERR_INVALID_ARGUMENT, "call dgpu_halo_setup first");
	if (c->ns)
		return fail(c, DGPU_ERR_UNSUPPORTED, "partitioned meshes: Euler and advection only");
	return DGPU_OK;
}

dgpu_status dgpu_halo_rhs_begin(dgpu_ctx* c)
{
	dgpu_status st = halo_ready(c);
	if (st != DGPU_OK || (st = ensure_coef(c)) != DGPU_OK)
		return st;
	DGPU_CUDA(c, c->launch_volume(c));
	DGPU_CUDA(c, launch_halo_copy(c, true));
	return DGPU_OK;
}

dgpu_status dgpu_halo_rhs_end(dgpu_ctx* c, double* max_rhs)
{
	dgpu_status st = halo_ready(c);
	if (st != DGPU_OK)
		return st;
	DGPU_CUDA(c, launch_halo_copy(c, false));
	DGPU_CUDA(c, c->launch_face(c));
	DGPU_CUDA(c, c->launch_lift_rhs(c));
	return read_max(c, max_rhs);
}

dgpu_status dgpu_halo_stage_begin(dgpu_ctx* c, int stage)
{
	dgpu_status st = halo_ready(c);
	if (st != DGPU_OK)
		return st;
	if (stage < 0 || stage > 2)
		return fail(c, DGPU_ERR_INVALID_ARGUMENT, "stage must be 0, 1 or 2");
	if (stage == 0 && (st = ensure_gl(c)) != DGPU_OK)
		return st;
	DGPU_CUDA(c, c->launch_volume_gl(c));
	DGPU_CUDA(c, launch_halo_copy(c, true));
	return DGPU_OK;
}

dgpu_status dgpu_halo_stage_end(dgpu_ctx* c, double dt, int stage, double* max_rhs)
{
	dgpu_status st = halo_ready(c);
	if (st != DGPU_OK)
		return st;
	if (stage < 0 || stage > 2 || !(dt == dt))
		return fail(c, DGPU_ERR_INVALID_ARGUMENT, "stage must be 0, 1 or 2 and dt a number");
	DGPU_CUDA(c, launch_halo_copy(c, false));
	DGPU_CUDA(c, c->launch_face(c));
	const bool want_max = (max_rhs != nullptr) && stage == 2;
	DGPU_CUDA(c, c->launch_lift_rk(c, dt, stage, want_max ? 1 : 0));
	if (stage == 2) {
		c->coef_valid = false;   // the current state is ug
		if (want_max && (st = read_max(c, max_rhs)) != DGPU_OK)
			return st;
		if (max_rhs && (st = check_positivity_flag(c)) != DGPU_OK)
			return st;
	}
	return DGPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------------------
// Source term (compute_source_rhs_dg_like, src/simulation/solvers/compute_rlhs.c:47-57)
// ---------------------------------------------------------------------------------------------------------------
extern "C" dgpu_status dgpu_set_source(dgpu_ctx* c, const double* source_vc)
{
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	const size_t n = state_size(c);
	if (!source_vc) {
		if (c->source) {
			DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
			cudaFree(c->source);
			c->source = nullptr;
			discard_graphs(c);
		}
		return DGPU_OK;
	}
	if (!c->source) {
		DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
		DGPU_CUDA(c, cudaMalloc((void**)&c->source, n * sizeof(double)));
		discard_graphs(c);   // captured steps hold the kernels' parameters, the source pointer among them
	}
	DGPU_CUDA(c, cudaMemcpyAsync(c->source, source_vc, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
	DGPU_CUDA(c, cudaStreamSynchronize(c->stream));
	return DGPU_OK;
}
