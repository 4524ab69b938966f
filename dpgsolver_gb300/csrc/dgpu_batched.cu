// C ABI of the batched (mixed element order) explicit DG residual: dgpu_batch_* in include/dgpu.h.
//
// Volumes are grouped by (element type, p) and stored group by group on the device; the caller's state stays in
// volume-list order and is permuted on upload/download. Each RK stage runs either as one launch per group and
// per face order ("plain") or as three persistent launches over all groups ("fused"), and a whole step is
// replayed from a captured CUDA graph. dgpu_batch_autotune times the elements-per-CTA candidates of every group
// and both forms on the actual mesh and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <stdio.h>
#include <string>
#include <vector>

#include "../../include/dgpu.h"
#include "dgpu_batched.cuh"
#include "dgpu_host_ops.h"

using namespace dgpu;

namespace {

thread_local std::string g_batch_error;

struct GroupLaunch {
	cudaError_t (*vol)(dgpu_batch*, int g, bool gll_in) = nullptr;
	cudaError_t (*lift)(dgpu_batch*, int g, int mode, double dt, int stage, int want_max) = nullptr;
	cudaError_t (*conv)(dgpu_batch*, int g, bool to_gl) = nullptr;
	int N = 0, E_max = 0;
};

}  // namespace

struct dgpu_batch {
	int d = 0, nv = 0, pde = 0, flux = 0, positivity = 0;
	double b_adv[3] = {0, 0, 0};
	int n_groups = 0, n_vol = 0, n_face = 0;
	std::vector<BGroup> hgroups;
	std::vector<BatchOps> hops;
	std::vector<GroupLaunch> gl;
	std::vector<int> order;            // sorted element -> list index
	std::vector<long long> list_off;   // list index -> offset in the caller's state
	std::vector<long long> sorted_off; // sorted element -> offset in the device state
	size_t ns = 0;
	// device
	BatchOps* d_ops = nullptr;
	BGroup* d_groups = nullptr;
	int4* d_elf = nullptr;
	long long* d_fbase = nullptr;
	double *gmet = nullptr, *inv_wJ = nullptr, *fgeo = nullptr;
	double *u = nullptr, *ug = nullptr, *u0 = nullptr, *rhs = nullptr, *vol_gl = nullptr;
	double *traces = nullptr, *nnf = nullptr;
	unsigned long long* max_bits = nullptr;
	int* err_flag = nullptr;
	unsigned long long* n_corr = nullptr;
	int* d_faces_by_q = nullptr;
	int* d_qf_begin = nullptr;
	int qf_begin[kQMax + 2] = {0};
	long long n_face_items = 0;
	BTile* d_tiles = nullptr;
	int n_tiles = 0, fused_blocks_vol = 0, fused_blocks_lift = 0, fused_blocks_face = 0;
	size_t fused_vol_smem = 0, fused_lift_smem = 0;
	cudaError_t (*fused_vol)(dgpu_batch*, bool gll_in) = nullptr;
	cudaError_t (*fused_lift)(dgpu_batch*, int mode, double dt, int stage, int want_max) = nullptr;
	cudaError_t (*fused_face)(dgpu_batch*) = nullptr;
	cudaError_t (*face_q)(dgpu_batch*, int qf) = nullptr;
	// execution
	cudaStream_t stream = nullptr;
	bool own_stream = false;
	bool coef_valid = true, gl_valid = false;
	int mode = 0;   // 0: one launch per group and face order; 1: fused persistent launches; 2: as 0 on parallel branches
	cudaStream_t aux[kQMax] = {nullptr};   // branches of form 2
	cudaEvent_t ev_fork = nullptr, ev_join[kQMax] = {nullptr};
	bool use_graphs = true;
	cudaGraphExec_t graph[3][2] = {};   // [mode][want_max]
	double graph_dt[3][2] = {};
	long long graph_launches[3][2] = {};   // kernels per replay
	long long launches = 0;
	std::string err;

	BParams params() const
	{
		BParams P;
		for (int k = 0; k < 3; ++k)
			P.b_adv[k] = b_adv[k];
		P.n_groups = n_groups;
		P.ops = d_ops;
		P.groups = d_groups;
		P.elf = d_elf;
		P.fbase = d_fbase;
		P.gmet = gmet;
		P.inv_wJ = inv_wJ;
		P.fgeo = fgeo;
		P.traces = traces;
		P.nnf = nnf;
		P.vol_gl = vol_gl;
		P.max_bits = max_bits;
		P.err_flag = err_flag;
		P.n_corr = n_corr;
		return P;
	}
};

namespace {

dgpu_status bfail(dgpu_batch* c, dgpu_status st, const std::string& m)
{
	if (c)
		c->err = m;
	else
		g_batch_error = m;
	return st;
}

#define BATCH_CUDA(ctx, call)                                                                              \
	do {                                                                                                   \
		cudaError_t e_ = (call);                                                                           \
		if (e_ != cudaSuccess)                                                                             \
			return bfail((ctx), DGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));        \
	} while (0)

template <int D, int Q, int NV>
size_t bvol_smem(int E) { return sizeof(BatchOps) + (size_t)E * BSmem<D, Q, NV>::VOL * sizeof(double); }
template <int D, int Q, int NV>
size_t blift_smem(int E) { return sizeof(BatchOps) + (size_t)E * BSmem<D, Q, NV>::LIFT * sizeof(double); }
template <int D, int Q, int NV>
size_t bconv_smem(int E) { return sizeof(BatchOps) + (size_t)E * 3 * NV * TPShape<D, Q>::N * sizeof(double); }

int threads_for(int E, int N) { return ((E * N + 31) / 32) * 32; }

template <int D, int Q, int NV, int PDE>
cudaError_t launch_bvol(dgpu_batch* c, int g, bool gll_in)
{
	const BGroup& G = c->hgroups[g];
	if (G.n_vol == 0)
		return cudaSuccess;
	const int blocks = (G.n_vol + G.E - 1) / G.E, thr = threads_for(G.E, TPShape<D, Q>::N);
	if (gll_in)
		bvol_group_kernel<D, Q, NV, PDE, true><<<blocks, thr, bvol_smem<D, Q, NV>(G.E), c->stream>>>(c->params(), g, c->u);
	else
		bvol_group_kernel<D, Q, NV, PDE, false><<<blocks, thr, bvol_smem<D, Q, NV>(G.E), c->stream>>>(c->params(), g, c->ug);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV>
cudaError_t launch_blift(dgpu_batch* c, int g, int mode, double dt, int stage, int want_max)
{
	const BGroup& G = c->hgroups[g];
	if (G.n_vol == 0)
		return cudaSuccess;
	const int blocks = (G.n_vol + G.E - 1) / G.E, thr = threads_for(G.E, TPShape<D, Q>::N);
	RkArgs rk;
	rk.u = c->ug;
	rk.u0 = c->u0;
	rk.rhs = c->rhs;
	rk.dt = dt;
	rk.stage = stage;
	rk.positivity = c->positivity;
	rk.want_max = want_max;
	if (mode == kModeRhs)
		blift_group_kernel<D, Q, NV, kModeRhs><<<blocks, thr, blift_smem<D, Q, NV>(G.E), c->stream>>>(c->params(), g, rk);
	else
		blift_group_kernel<D, Q, NV, kModeRkGl><<<blocks, thr, blift_smem<D, Q, NV>(G.E), c->stream>>>(c->params(), g, rk);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV>
cudaError_t launch_bconv(dgpu_batch* c, int g, bool to_gl)
{
	const BGroup& G = c->hgroups[g];
	if (G.n_vol == 0)
		return cudaSuccess;
	const int blocks = (G.n_vol + G.E - 1) / G.E, thr = threads_for(G.E, TPShape<D, Q>::N);
	if (to_gl)
		bconvert_group_kernel<D, Q, NV, true><<<blocks, thr, bconv_smem<D, Q, NV>(G.E), c->stream>>>(c->params(), g, c->u, c->ug);
	else
		bconvert_group_kernel<D, Q, NV, false><<<blocks, thr, bconv_smem<D, Q, NV>(G.E), c->stream>>>(c->params(), g, c->ug, c->u);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int NV, int PDE, int FLUX>
cudaError_t launch_bface_q(dgpu_batch* c, int qf)
{
	const int n = c->qf_begin[qf + 1] - c->qf_begin[qf];
	if (n == 0)
		return cudaSuccess;
	const int* faces = c->d_faces_by_q + c->qf_begin[qf];
	const long long items = (long long)n * (D == 2 ? qf : qf * qf);
	const unsigned blocks = (unsigned)((items + 255) / 256);
	switch (qf) {
	case 2: bface_group_kernel<D, 2, NV, PDE, FLUX><<<blocks, 256, 0, c->stream>>>(c->params(), faces, n); break;
	case 3: bface_group_kernel<D, 3, NV, PDE, FLUX><<<blocks, 256, 0, c->stream>>>(c->params(), faces, n); break;
	case 4: bface_group_kernel<D, 4, NV, PDE, FLUX><<<blocks, 256, 0, c->stream>>>(c->params(), faces, n); break;
	default: bface_group_kernel<D, 5, NV, PDE, FLUX><<<blocks, 256, 0, c->stream>>>(c->params(), faces, n); break;
	}
	c->launches++;
	return cudaGetLastError();
}

template <int D, int NV, int PDE>
cudaError_t launch_fused_vol(dgpu_batch* c, bool gll_in)
{
	if (gll_in)
		bvol_fused_kernel<D, NV, PDE, true><<<c->fused_blocks_vol, 256, c->fused_vol_smem, c->stream>>>(
			c->params(), c->d_tiles, c->n_tiles, c->u);
	else
		bvol_fused_kernel<D, NV, PDE, false><<<c->fused_blocks_vol, 256, c->fused_vol_smem, c->stream>>>(
			c->params(), c->d_tiles, c->n_tiles, c->ug);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int NV>
cudaError_t launch_fused_lift(dgpu_batch* c, int mode, double dt, int stage, int want_max)
{
	RkArgs rk;
	rk.u = c->ug;
	rk.u0 = c->u0;
	rk.rhs = c->rhs;
	rk.dt = dt;
	rk.stage = stage;
	rk.positivity = c->positivity;
	rk.want_max = want_max;
	if (mode == kModeRhs)
		blift_fused_kernel<D, NV, kModeRhs><<<c->fused_blocks_lift, 256, c->fused_lift_smem, c->stream>>>(
			c->params(), c->d_tiles, c->n_tiles, rk);
	else
		blift_fused_kernel<D, NV, kModeRkGl><<<c->fused_blocks_lift, 256, c->fused_lift_smem, c->stream>>>(
			c->params(), c->d_tiles, c->n_tiles, rk);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int NV, int PDE, int FLUX>
cudaError_t launch_fused_face(dgpu_batch* c)
{
	bface_fused_kernel<D, NV, PDE, FLUX><<<c->fused_blocks_face, 256, 0, c->stream>>>(
		c->params(), c->d_faces_by_q, c->d_qf_begin, c->n_face_items);
	c->launches++;
	return cudaGetLastError();
}

template <int D, int Q, int NV, int PDE>
cudaError_t bind_group(dgpu_batch* c, int g)
{
	GroupLaunch& L = c->gl[g];
	L.vol = launch_bvol<D, Q, NV, PDE>;
	L.lift = launch_blift<D, Q, NV>;
	L.conv = launch_bconv<D, Q, NV>;
	L.N = TPShape<D, Q>::N;
	L.E_max = std::max(1, 256 / L.N);
	const cudaFuncAttribute A = cudaFuncAttributeMaxDynamicSharedMemorySize;
	const int E = L.E_max;
	cudaError_t e;
	if ((e = cudaFuncSetAttribute(bvol_group_kernel<D, Q, NV, PDE, true>, A, (int)bvol_smem<D, Q, NV>(E))))
		return e;
	if ((e = cudaFuncSetAttribute(bvol_group_kernel<D, Q, NV, PDE, false>, A, (int)bvol_smem<D, Q, NV>(E))))
		return e;
	if ((e = cudaFuncSetAttribute(blift_group_kernel<D, Q, NV, kModeRhs>, A, (int)blift_smem<D, Q, NV>(E))))
		return e;
	if ((e = cudaFuncSetAttribute(blift_group_kernel<D, Q, NV, kModeRkGl>, A, (int)blift_smem<D, Q, NV>(E))))
		return e;
	if ((e = cudaFuncSetAttribute(bconvert_group_kernel<D, Q, NV, true>, A, (int)bconv_smem<D, Q, NV>(E))))
		return e;
	if ((e = cudaFuncSetAttribute(bconvert_group_kernel<D, Q, NV, false>, A, (int)bconv_smem<D, Q, NV>(E))))
		return e;
	// the fused kernels need the largest of the groups' shared memory
	c->fused_vol_smem = std::max(c->fused_vol_smem, bvol_smem<D, Q, NV>(E));
	c->fused_lift_smem = std::max(c->fused_lift_smem, blift_smem<D, Q, NV>(E));
	return cudaSuccess;
}

template <int D, int NV, int PDE>
cudaError_t bind_groups_q(dgpu_batch* c)
{
	for (int g = 0; g < c->n_groups; ++g) {
		cudaError_t e;
		switch (c->hgroups[g].q) {
		case 2: e = bind_group<D, 2, NV, PDE>(c, g); break;
		case 3: e = bind_group<D, 3, NV, PDE>(c, g); break;
		case 4: e = bind_group<D, 4, NV, PDE>(c, g); break;
		default: e = bind_group<D, 5, NV, PDE>(c, g); break;
		}
		if (e != cudaSuccess)
			return e;
	}
	return cudaSuccess;
}

template <int D, int NV, int PDE, int FLUX>
cudaError_t bind_all(dgpu_batch* c)
{
	cudaError_t e = bind_groups_q<D, NV, PDE>(c);
	if (e != cudaSuccess)
		return e;
	c->fused_vol = launch_fused_vol<D, NV, PDE>;
	c->fused_lift = launch_fused_lift<D, NV>;
	c->fused_face = launch_fused_face<D, NV, PDE, FLUX>;
	c->face_q = launch_bface_q<D, NV, PDE, FLUX>;
	const cudaFuncAttribute A = cudaFuncAttributeMaxDynamicSharedMemorySize;
	if ((e = cudaFuncSetAttribute(bvol_fused_kernel<D, NV, PDE, true>, A, (int)c->fused_vol_smem)))
		return e;
	if ((e = cudaFuncSetAttribute(bvol_fused_kernel<D, NV, PDE, false>, A, (int)c->fused_vol_smem)))
		return e;
	if ((e = cudaFuncSetAttribute(blift_fused_kernel<D, NV, kModeRhs>, A, (int)c->fused_lift_smem)))
		return e;
	if ((e = cudaFuncSetAttribute(blift_fused_kernel<D, NV, kModeRkGl>, A, (int)c->fused_lift_smem)))
		return e;
	// persistent grids: as many CTAs as fit on the device at once
	int dev = 0, sms = 0, per_sm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bvol_fused_kernel<D, NV, PDE, false>, 256, c->fused_vol_smem);
	c->fused_blocks_vol = std::max(1, std::min(c->n_tiles, sms * std::max(1, per_sm)));
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, blift_fused_kernel<D, NV, kModeRkGl>, 256, c->fused_lift_smem);
	c->fused_blocks_lift = std::max(1, std::min(c->n_tiles, sms * std::max(1, per_sm)));
	c->fused_blocks_face = (int)std::max<long long>(1, std::min<long long>((c->n_face_items + 255) / 256, (long long)sms * 8));
	return cudaGetLastError();
}

cudaError_t bind(dgpu_batch* c)
{
	if (c->d == 2) {
		if (c->pde == DGPU_PDE_ADVECTION) return bind_all<2, 1, kAdvection, kUpwind>(c);
		if (c->flux == DGPU_NUM_FLUX_ROE_PIKE) return bind_all<2, 4, kEuler, kRoePike>(c);
		return bind_all<2, 4, kEuler, kLaxFriedrichs>(c);
	}
	if (c->pde == DGPU_PDE_ADVECTION) return bind_all<3, 1, kAdvection, kUpwind>(c);
	if (c->flux == DGPU_NUM_FLUX_ROE_PIKE) return bind_all<3, 5, kEuler, kRoePike>(c);
	return bind_all<3, 5, kEuler, kLaxFriedrichs>(c);
}

void free_batch(dgpu_batch* c)
{
	for (auto& gm : c->graph)
		for (auto& g : gm)
			if (g)
				cudaGraphExecDestroy(g);
	void* ptrs[] = {c->d_ops, c->d_groups, c->d_elf, c->d_fbase, c->gmet, c->inv_wJ, c->fgeo, c->u, c->ug, c->u0,
	                c->rhs, c->vol_gl, c->traces, c->nnf, c->max_bits, c->err_flag, c->n_corr, c->d_faces_by_q,
	                c->d_qf_begin, c->d_tiles};
	for (void* p : ptrs)
		if (p)
			cudaFree(p);
	if (c->own_stream && c->stream)
		cudaStreamDestroy(c->stream);
	for (int j = 0; j < kQMax; ++j) {
		if (c->aux[j])
			cudaStreamDestroy(c->aux[j]);
		if (c->ev_join[j])
			cudaEventDestroy(c->ev_join[j]);
	}
	if (c->ev_fork)
		cudaEventDestroy(c->ev_fork);
}

template <typename T>
cudaError_t upload_vec(T** dst, const std::vector<T>& src)
{
	cudaError_t e = cudaMalloc((void**)dst, std::max<size_t>(1, src.size()) * sizeof(T));
	if (e != cudaSuccess || src.empty())
		return e;
	return cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
}

// Form 2: the calls of `launch(j, i)` for i in items run on the branch streams, forked from and joined back into
// the context's stream (under stream capture: parallel branches of the graph).
template <typename F>
dgpu_status on_branches(dgpu_batch* c, int n_items, F launch)
{
	cudaStream_t main = c->stream;
	BATCH_CUDA(c, cudaEventRecord(c->ev_fork, main));
	int j = 0;
	for (int i = 0; i < n_items; ++i) {
		cudaStream_t br = c->aux[j];
		BATCH_CUDA(c, cudaStreamWaitEvent(br, c->ev_fork, 0));
		c->stream = br;
		const long long before = c->launches;
		cudaError_t e = launch(i);
		c->stream = main;
		BATCH_CUDA(c, e);
		if (c->launches == before)   // nothing launched (empty group or face order): no branch
			continue;
		BATCH_CUDA(c, cudaEventRecord(c->ev_join[j], br));
		BATCH_CUDA(c, cudaStreamWaitEvent(main, c->ev_join[j], 0));
		++j;
	}
	return DGPU_OK;
}

// One residual on GLL coefficients, or one RK stage on GL nodal values.
dgpu_status enqueue_stage(dgpu_batch* c, bool rhs_mode, double dt, int stage, int want_max)
{
	const int lmode = rhs_mode ? kModeRhs : kModeRkGl;
	if (c->mode == 1) {
		BATCH_CUDA(c, c->fused_vol(c, rhs_mode));
		BATCH_CUDA(c, c->fused_face(c));
		BATCH_CUDA(c, c->fused_lift(c, lmode, dt, stage, want_max));
	} else if (c->mode == 2) {
		dgpu_status st;
		if ((st = on_branches(c, c->n_groups, [&](int g) { return c->gl[g].vol(c, g, rhs_mode); })) != DGPU_OK)
			return st;
		if ((st = on_branches(c, kQMax - 1, [&](int i) { return c->face_q(c, i + 2); })) != DGPU_OK)
			return st;
		if ((st = on_branches(c, c->n_groups,
		                      [&](int g) { return c->gl[g].lift(c, g, lmode, dt, stage, want_max); })) != DGPU_OK)
			return st;
	} else {
		for (int g = 0; g < c->n_groups; ++g)
			BATCH_CUDA(c, c->gl[g].vol(c, g, rhs_mode));
		for (int qf = 2; qf <= kQMax; ++qf)
			BATCH_CUDA(c, c->face_q(c, qf));
		for (int g = 0; g < c->n_groups; ++g)
			BATCH_CUDA(c, c->gl[g].lift(c, g, lmode, dt, stage, want_max));
	}
	return DGPU_OK;
}

dgpu_status ensure_coef(dgpu_batch* c)
{
	if (!c->coef_valid) {
		for (int g = 0; g < c->n_groups; ++g)
			BATCH_CUDA(c, c->gl[g].conv(c, g, false));
		c->coef_valid = true;
	}
	return DGPU_OK;
}

dgpu_status ensure_gl(dgpu_batch* c)
{
	if (!c->gl_valid) {
		for (int g = 0; g < c->n_groups; ++g)
			BATCH_CUDA(c, c->gl[g].conv(c, g, true));
		c->gl_valid = true;
	}
	return DGPU_OK;
}

dgpu_status read_max(dgpu_batch* c, double* max_rhs)
{
	if (!max_rhs)
		return DGPU_OK;
	unsigned long long bits = 0;
	BATCH_CUDA(c, cudaMemcpyAsync(&bits, c->max_bits, sizeof bits, cudaMemcpyDeviceToHost, c->stream));
	BATCH_CUDA(c, cudaStreamSynchronize(c->stream));
	memcpy(max_rhs, &bits, sizeof(double));
	return DGPU_OK;
}

void drop_graphs(dgpu_batch* c)
{
	for (auto& gm : c->graph)
		for (auto& g : gm)
			if (g) {
				cudaGraphExecDestroy(g);
				g = nullptr;
			}
}

}  // namespace

extern "C" {

dgpu_status dgpu_batch_create(const dgpu_physics* phys, int n_groups, const dgpu_tp_operators* ops,
                              const int* vol_group, const dgpu_mesh* mesh, dgpu_batch** out)
{
	g_batch_error.clear();
	if (!phys || n_groups < 1 || !ops || !vol_group || !mesh || !out)
		return bfail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "NULL argument");
	*out = nullptr;
	const int d = phys->d;
	if (d != 2 && d != 3)
		return bfail(nullptr, DGPU_ERR_UNSUPPORTED, "d must be 2 or 3");
	if (phys->pde == DGPU_PDE_ADVECTION ? phys->num_flux != DGPU_NUM_FLUX_UPWIND
	                                    : (phys->pde != DGPU_PDE_EULER ||
	                                       (phys->num_flux != DGPU_NUM_FLUX_ROE_PIKE &&
	                                        phys->num_flux != DGPU_NUM_FLUX_LAX_FRIEDRICHS)))
		return bfail(nullptr, DGPU_ERR_UNSUPPORTED, "advection/upwind or Euler/Roe-Pike/Lax-Friedrichs only");
	if (mesh->n_volumes < 1 || mesh->n_faces < 1 || !mesh->metrics_vc || !mesh->jacobian_det_vc ||
	    !mesh->face_vol || !mesh->face_lf || !mesh->normals_fc || !mesh->jacobian_det_fc)
		return bfail(nullptr, DGPU_ERR_INVALID_ARGUMENT, "incomplete mesh");
	int dev = 0, n_dev = 0;
	if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev < 1)
		return bfail(nullptr, DGPU_ERR_NO_DEVICE, "no CUDA device");
	cudaGetDevice(&dev);
	cudaDeviceProp prop;
	if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || prop.major * 10 + prop.minor != 103)
		return bfail(nullptr, DGPU_ERR_NO_DEVICE, "device is not compute capability 10.3 (sm_103a build)");

	dgpu_batch* c = new dgpu_batch();
	c->d = d;
	c->pde = phys->pde;
	c->flux = phys->num_flux;
	c->nv = (phys->pde == DGPU_PDE_EULER ? d + 2 : 1);
	c->positivity = (phys->pde == DGPU_PDE_EULER && phys->positivity) ? 1 : 0;
	for (int k = 0; k < 3; ++k)
		c->b_adv[k] = phys->b_adv[k];
	c->n_groups = n_groups;
	c->n_vol = mesh->n_volumes;
	c->n_face = mesh->n_faces;
	const int nv = c->nv, nV = c->n_vol, nF = c->n_face;
	auto reject = [&](dgpu_status st, const char* m) {
		delete c;
		return bfail(nullptr, st, m);
	};

	// ---- groups and their operators ----
	c->hgroups.resize(n_groups);
	c->hops.resize(n_groups);
	std::vector<std::vector<double>> w(n_groups);
	for (int g = 0; g < n_groups; ++g) {
		const dgpu_tp_operators& o = ops[g];
		if ((d == 2 && o.elem_type != DGPU_QUAD) || (d == 3 && o.elem_type != DGPU_HEX) || o.p < 1 || o.p > kQMax - 1)
			return reject(DGPU_ERR_UNSUPPORTED, "groups must be QUAD (d=2) or HEX (d=3) with p in 1..4");
		if (!o.cv0_vs_vc || !o.cv1_vs_vc || !o.cv0_vs_fc || !o.w_vc)
			return reject(DGPU_ERR_INVALID_ARGUMENT, "NULL operator");
		if (c->positivity && (!o.ccSB0_vs_vs || !o.ccBS0_vs_vs))
			return reject(DGPU_ERR_INVALID_ARGUMENT, "positivity needs ccSB0/ccBS0");
		const int q = o.p + 1;
		for (int h = 0; h < g; ++h)
			if (c->hgroups[h].q == q)
				return reject(DGPU_ERR_INVALID_ARGUMENT, "two groups with the same p");
		memset(&c->hops[g], 0, sizeof(BatchOps));
		if (!derive_tp_ops(&o, d, &c->hops[g].t))
			return reject(DGPU_ERR_INVALID_ARGUMENT, "cv0_vs_vc is singular");
		// GL(q) Lagrange at GL(qf) nodes for every face order qf >= q
		double xq[kQMax], xf[kQMax];
		gauss_legendre_nodes(q, xq);
		for (int qf = q; qf <= kQMax; ++qf) {
			gauss_legendre_nodes(qf, xf);
			for (int i = 0; i < qf; ++i)
				for (int a = 0; a < q; ++a)
					c->hops[g].Iup[qf][i][a] = lagrange_value(xq, q, a, xf[i]);
		}
		c->hgroups[g].q = q;
		const int N = (d == 2 ? q * q : q * q * q);
		w[g].resize(N);
		for (int n = 0; n < N; ++n) {
			int r = n;
			double x = 1.0;
			for (int k = 0; k < d; ++k) {
				x *= o.w_vc[r % q];
				r /= q;
			}
			w[g][n] = x;
		}
	}
	// ---- volumes: group-sorted order, offsets ----
	std::vector<int> count(n_groups, 0);
	for (int v = 0; v < nV; ++v) {
		if (vol_group[v] < 0 || vol_group[v] >= n_groups)
			return reject(DGPU_ERR_INVALID_ARGUMENT, "vol_group out of range");
		count[vol_group[v]]++;
	}
	c->list_off.resize(nV + 1);
	std::vector<long long> list_vc_off(nV + 1);
	long long so = 0, vco = 0;
	for (int v = 0; v < nV; ++v) {
		const int q = c->hgroups[vol_group[v]].q, N = (d == 2 ? q * q : q * q * q);
		c->list_off[v] = so;
		list_vc_off[v] = vco;
		so += (long long)nv * N;
		vco += N;
	}
	c->list_off[nV] = so;
	c->ns = (size_t)so;
	c->order.resize(nV);
	std::vector<int> sorted_pos(nV);
	{
		long long elem = 0, st_off = 0, gm_off = 0, wj_off = 0;
		std::vector<int> next(n_groups);
		for (int g = 0; g < n_groups; ++g) {
			const int q = c->hgroups[g].q, N = (d == 2 ? q * q : q * q * q);
			BGroup& G = c->hgroups[g];
			G.n_vol = count[g];
			G.elem0 = elem;
			G.state_off = st_off;
			G.gmet_off = gm_off;
			G.wj_off = wj_off;
			G.E = std::max(1, 256 / N);
			next[g] = (int)elem;
			elem += count[g];
			st_off += (long long)count[g] * nv * N;
			gm_off += (long long)count[g] * d * d * N;
			wj_off += (long long)count[g] * N;
		}
		for (int v = 0; v < nV; ++v) {
			const int p = next[vol_group[v]]++;
			c->order[p] = v;
			sorted_pos[v] = p;
		}
	}
	c->sorted_off.resize(nV);
	std::vector<double> gmet, inv_wJ;
	for (int g = 0; g < n_groups; ++g) {
		const int q = c->hgroups[g].q, N = (d == 2 ? q * q : q * q * q);
		for (int e = 0; e < c->hgroups[g].n_vol; ++e) {
			const int p = (int)c->hgroups[g].elem0 + e, v = c->order[p];
			c->sorted_off[p] = c->hgroups[g].state_off + (long long)e * nv * N;
			const double* m = mesh->metrics_vc + list_vc_off[v] * d * d;
			const double* J = mesh->jacobian_det_vc + list_vc_off[v];
			for (int j = 0; j < d; ++j)
				for (int i = 0; i < d; ++i)
					for (int n = 0; n < N; ++n)
						gmet.push_back(w[g][n] * m[n + (size_t)N * (i + d * j)]);
			for (int n = 0; n < N; ++n) {
				if (!(J[n] > 0.0))
					return reject(DGPU_ERR_INVALID_ARGUMENT, "non-positive jacobian_det_vc");
				inv_wJ.push_back(1.0 / (w[g][n] * J[n]));
			}
		}
	}
	// ---- faces: order p_f = max of the sides, face data at its q_f points ----
	std::vector<int> face_q(nF);
	std::vector<long long> fbase(nF + 1);
	std::vector<int4> elf((size_t)nV * 2 * d, int4{-1, -1, -1, 0});
	long long fb = 0;
	for (int f = 0; f < nF; ++f) {
		int qf = 0;
		for (int s = 0; s < 2; ++s) {
			const int v = mesh->face_vol[2 * f + s], lf = mesh->face_lf[2 * f + s];
			if (v < 0)
				return reject(DGPU_ERR_UNSUPPORTED, "boundary faces are not supported (periodic meshes)");
			if (v >= nV || lf < 0 || lf >= 2 * d)
				return reject(DGPU_ERR_INVALID_ARGUMENT, "bad face connectivity");
			qf = std::max(qf, c->hgroups[vol_group[v]].q);
		}
		face_q[f] = qf;
		fbase[f] = fb;
		const int nff = (d == 2 ? qf : qf * qf);
		fb += nff;
		for (int s = 0; s < 2; ++s) {
			const int v = mesh->face_vol[2 * f + s], lf = mesh->face_lf[2 * f + s];
			int4& slot = elf[(size_t)sorted_pos[v] * 2 * d + lf];
			if (slot.x != -1)
				return reject(DGPU_ERR_INVALID_ARGUMENT, "a volume face appears twice in the face list");
			slot = int4{f, s, qf, 0};
		}
		if (mesh->nc_fc)
			for (int i = 0; i < nff; ++i)
				if (mesh->nc_fc[fbase[f] + i] != i)
					return reject(DGPU_ERR_UNSUPPORTED, "the batched path needs aligned faces (identity nc_fc)");
	}
	fbase[nF] = fb;
	for (size_t i = 0; i < elf.size(); ++i)
		if (elf[i].x < 0)
			return reject(DGPU_ERR_INVALID_ARGUMENT, "a volume face is missing from the face list");
	// face weights: q_f is always the q of one of the groups, whose GL weights the caller gave
	double wq[kQMax + 1][kQMax] = {{0}};
	for (int g = 0; g < n_groups; ++g)
		for (int a = 0; a < c->hgroups[g].q; ++a)
			wq[c->hgroups[g].q][a] = ops[g].w_vc[a];
	std::vector<double> fgeo((size_t)(d + 1) * fb);
	for (int f = 0; f < nF; ++f) {
		const int qf = face_q[f], nff = (d == 2 ? qf : qf * qf);
		for (int i = 0; i < nff; ++i) {
			const double wf = (d == 2 ? wq[qf][i] : wq[qf][i % qf] * wq[qf][i / qf]);
			for (int k = 0; k < d; ++k)
				fgeo[(d + 1) * fbase[f] + (size_t)k * nff + i] = mesh->normals_fc[(fbase[f] + i) * d + k];
			fgeo[(d + 1) * fbase[f] + (size_t)d * nff + i] = wf * mesh->jacobian_det_fc[fbase[f] + i];
		}
	}
	std::vector<int> faces_by_q;
	for (int qf = 0; qf <= kQMax + 1; ++qf)
		c->qf_begin[qf] = 0;
	for (int qf = 2; qf <= kQMax; ++qf) {
		c->qf_begin[qf] = (int)faces_by_q.size();
		for (int f = 0; f < nF; ++f)
			if (face_q[f] == qf)
				faces_by_q.push_back(f);
	}
	c->qf_begin[kQMax + 1] = (int)faces_by_q.size();
	c->n_face_items = 0;
	for (int qf = 2; qf <= kQMax; ++qf)
		c->n_face_items += (long long)(c->qf_begin[qf + 1] - c->qf_begin[qf]) * (d == 2 ? qf : qf * qf);
	// fused tiles: full CTAs of 256 threads per group
	std::vector<BTile> tiles;
	for (int g = 0; g < n_groups; ++g) {
		const int q = c->hgroups[g].q, N = (d == 2 ? q * q : q * q * q), E = std::max(1, 256 / N);
		c->hgroups[g].first_tile = (int)tiles.size();
		for (int e0 = 0; e0 < c->hgroups[g].n_vol; e0 += E)
			tiles.push_back(BTile{g, e0});
	}
	c->n_tiles = (int)tiles.size();

	// ---- device ----
#define B_TRY(call)                                                                                  \
	do {                                                                                             \
		cudaError_t e_ = (call);                                                                     \
		if (e_ != cudaSuccess) {                                                                     \
			std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_);                     \
			free_batch(c);                                                                           \
			delete c;                                                                                \
			return bfail(nullptr, DGPU_ERR_CUDA, m_);                                                \
		}                                                                                            \
	} while (0)
	B_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
	c->own_stream = true;
	for (int j = 0; j < kQMax; ++j) {
		B_TRY(cudaStreamCreateWithFlags(&c->aux[j], cudaStreamNonBlocking));
		B_TRY(cudaEventCreateWithFlags(&c->ev_join[j], cudaEventDisableTiming));
	}
	B_TRY(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
	const size_t ns = c->ns;
	B_TRY(cudaMalloc((void**)&c->u, ns * sizeof(double)));
	B_TRY(cudaMalloc((void**)&c->ug, ns * sizeof(double)));
	B_TRY(cudaMalloc((void**)&c->u0, ns * sizeof(double)));
	B_TRY(cudaMalloc((void**)&c->rhs, ns * sizeof(double)));
	B_TRY(cudaMalloc((void**)&c->vol_gl, ns * sizeof(double)));
	B_TRY(cudaMalloc((void**)&c->traces, (size_t)2 * nv * fb * sizeof(double)));
	B_TRY(cudaMalloc((void**)&c->nnf, (size_t)nv * fb * sizeof(double)));
	B_TRY(cudaMalloc((void**)&c->max_bits, sizeof(unsigned long long)));
	B_TRY(cudaMalloc((void**)&c->err_flag, sizeof(int)));
	B_TRY(cudaMalloc((void**)&c->n_corr, sizeof(unsigned long long)));
	B_TRY(cudaMemset(c->u, 0, ns * sizeof(double)));
	B_TRY(cudaMemset(c->traces, 0, (size_t)2 * nv * fb * sizeof(double)));
	B_TRY(cudaMemset(c->nnf, 0, (size_t)nv * fb * sizeof(double)));
	B_TRY(cudaMemset(c->max_bits, 0, sizeof(unsigned long long)));
	B_TRY(cudaMemset(c->err_flag, 0, sizeof(int)));
	B_TRY(cudaMemset(c->n_corr, 0, sizeof(unsigned long long)));
	B_TRY(upload_vec(&c->d_ops, c->hops));
	B_TRY(upload_vec(&c->d_groups, c->hgroups));
	B_TRY(upload_vec(&c->d_elf, elf));
	B_TRY(upload_vec(&c->d_fbase, fbase));
	B_TRY(upload_vec(&c->gmet, gmet));
	B_TRY(upload_vec(&c->inv_wJ, inv_wJ));
	B_TRY(upload_vec(&c->fgeo, fgeo));
	B_TRY(upload_vec(&c->d_faces_by_q, faces_by_q));
	std::vector<int> qb(c->qf_begin, c->qf_begin + kQMax + 2);
	B_TRY(upload_vec(&c->d_qf_begin, qb));
	B_TRY(upload_vec(&c->d_tiles, tiles));
	c->gl.resize(n_groups);
	B_TRY(bind(c));
#undef B_TRY
	*out = c;
	return DGPU_OK;
}

dgpu_status dgpu_batch_destroy(dgpu_batch* c)
{
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	if (c->stream)
		cudaStreamSynchronize(c->stream);
	free_batch(c);
	delete c;
	return DGPU_OK;
}

const char* dgpu_batch_last_error(const dgpu_batch* c) { return c ? c->err.c_str() : g_batch_error.c_str(); }

dgpu_status dgpu_batch_state_size(const dgpu_batch* c, size_t* n)
{
	if (!c || !n)
		return DGPU_ERR_INVALID_ARGUMENT;
	*n = c->ns;
	return DGPU_OK;
}

dgpu_status dgpu_batch_upload_state(dgpu_batch* c, const double* sol)
{
	if (!c || !sol)
		return DGPU_ERR_INVALID_ARGUMENT;
	std::vector<double> h(c->ns);
	for (int p = 0; p < c->n_vol; ++p) {
		const int v = c->order[p];
		std::copy(sol + c->list_off[v], sol + c->list_off[v + 1], h.begin() + c->sorted_off[p]);
	}
	BATCH_CUDA(c, cudaMemcpyAsync(c->u, h.data(), c->ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
	BATCH_CUDA(c, cudaStreamSynchronize(c->stream));
	c->coef_valid = true;
	c->gl_valid = false;
	return DGPU_OK;
}

static dgpu_status download_perm(dgpu_batch* c, const double* dev, double* sol)
{
	std::vector<double> h(c->ns);
	BATCH_CUDA(c, cudaMemcpyAsync(h.data(), dev, c->ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
	BATCH_CUDA(c, cudaStreamSynchronize(c->stream));
	for (int p = 0; p < c->n_vol; ++p) {
		const int v = c->order[p];
		std::copy(h.begin() + c->sorted_off[p], h.begin() + c->sorted_off[p] + (c->list_off[v + 1] - c->list_off[v]),
		          sol + c->list_off[v]);
	}
	return DGPU_OK;
}

dgpu_status dgpu_batch_download_state(dgpu_batch* c, double* sol)
{
	if (!c || !sol)
		return DGPU_ERR_INVALID_ARGUMENT;
	dgpu_status st = ensure_coef(c);
	if (st != DGPU_OK)
		return st;
	return download_perm(c, c->u, sol);
}

dgpu_status dgpu_batch_download_rhs(dgpu_batch* c, double* rhs)
{
	if (!c || !rhs)
		return DGPU_ERR_INVALID_ARGUMENT;
	return download_perm(c, c->rhs, rhs);
}

dgpu_status dgpu_batch_compute_rhs(dgpu_batch* c, double* max_rhs)
{
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	dgpu_status st = ensure_coef(c);
	if (st != DGPU_OK)
		return st;
	if ((st = enqueue_stage(c, true, 0.0, 0, 1)) != DGPU_OK)
		return st;
	return read_max(c, max_rhs);
}

dgpu_status dgpu_batch_ssp_rk3_steps(dgpu_batch* c, double dt, int n_steps, double* max_rhs)
{
	if (!c || n_steps < 0 || !(dt == dt))
		return DGPU_ERR_INVALID_ARGUMENT;
	dgpu_status st = ensure_gl(c);
	if (st != DGPU_OK)
		return st;
	const int wm = max_rhs ? 1 : 0;
	for (int s = 0; s < n_steps; ++s) {
		const int want = (wm && s == n_steps - 1) ? 1 : 0;
		if (!c->use_graphs) {
			for (int stage = 0; stage < 3 && st == DGPU_OK; ++stage)
				st = enqueue_stage(c, false, dt, stage, (want && stage == 2) ? 1 : 0);
			if (st != DGPU_OK)
				return st;
			continue;
		}
		cudaGraphExec_t& gx = c->graph[c->mode][want];
		if (!gx || c->graph_dt[c->mode][want] != dt) {
			if (gx) {
				cudaGraphExecDestroy(gx);
				gx = nullptr;
			}
			cudaGraph_t g;
			BATCH_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
			const long long before = c->launches;
			for (int stage = 0; stage < 3 && st == DGPU_OK; ++stage)
				st = enqueue_stage(c, false, dt, stage, (want && stage == 2) ? 1 : 0);
			c->graph_launches[c->mode][want] = c->launches - before;
			c->launches = before;
			cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
			if (st != DGPU_OK)
				return st;
			BATCH_CUDA(c, ec);
			cudaError_t ei = cudaGraphInstantiate(&gx, g, 0);
			cudaGraphDestroy(g);
			BATCH_CUDA(c, ei);
			c->graph_dt[c->mode][want] = dt;
		}
		BATCH_CUDA(c, cudaGraphLaunch(gx, c->stream));
		c->launches += c->graph_launches[c->mode][want];
	}
	if (n_steps > 0)
		c->coef_valid = false;
	if (c->positivity) {
		int flag = 0;
		BATCH_CUDA(c, cudaMemcpyAsync(&flag, c->err_flag, sizeof flag, cudaMemcpyDeviceToHost, c->stream));
		BATCH_CUDA(c, cudaStreamSynchronize(c->stream));
		if (flag)
			return bfail(c, DGPU_ERR_POSITIVITY, "average density or pressure below EPS_PHYS");
	}
	return read_max(c, max_rhs);
}

dgpu_status dgpu_batch_set_mode(dgpu_batch* c, int form)
{
	if (!c || form < 0 || form > 2)
		return DGPU_ERR_INVALID_ARGUMENT;
	c->mode = form;
	return DGPU_OK;
}

dgpu_status dgpu_batch_set_group_tile(dgpu_batch* c, int group, int elements_per_cta)
{
	if (!c || group < 0 || group >= c->n_groups || elements_per_cta < 1 || elements_per_cta > c->gl[group].E_max)
		return DGPU_ERR_INVALID_ARGUMENT;
	c->hgroups[group].E = elements_per_cta;
	BATCH_CUDA(c, cudaMemcpyAsync(c->d_groups, c->hgroups.data(), c->hgroups.size() * sizeof(BGroup),
	                              cudaMemcpyHostToDevice, c->stream));
	BATCH_CUDA(c, cudaStreamSynchronize(c->stream));
	drop_graphs(c);
	return DGPU_OK;
}

dgpu_status dgpu_batch_autotune(dgpu_batch* c, double dt, int reps, char* report, size_t report_len)
{
	if (!c || reps < 1 || !(dt == dt))
		return DGPU_ERR_INVALID_ARGUMENT;
	std::string rep;
	// keep the state, the residual and the correction count: tuning runs steps and residuals on them
	const bool coef_was = c->coef_valid, gl_was = c->gl_valid;
	double* saved = nullptr;
	unsigned long long n_corr0 = 0;
	BATCH_CUDA(c, cudaMalloc((void**)&saved, 2 * c->ns * sizeof(double)));
	BATCH_CUDA(c, cudaMemcpyAsync(saved, coef_was ? c->u : c->ug, c->ns * sizeof(double), cudaMemcpyDeviceToDevice,
	                              c->stream));
	BATCH_CUDA(c, cudaMemcpyAsync(saved + c->ns, c->rhs, c->ns * sizeof(double), cudaMemcpyDeviceToDevice,
	                              c->stream));
	BATCH_CUDA(c, cudaMemcpyAsync(&n_corr0, c->n_corr, sizeof n_corr0, cudaMemcpyDeviceToHost, c->stream));
	BATCH_CUDA(c, cudaStreamSynchronize(c->stream));
	dgpu_status st = ensure_gl(c);
	if (st != DGPU_OK) {
		cudaFree(saved);
		return st;
	}
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	auto time_group = [&](int g) -> float {
		float best = 0.f;
		for (int r = 0; r < reps + 1; ++r) {
			cudaEventRecord(e0, c->stream);
			c->gl[g].vol(c, g, false);
			c->gl[g].lift(c, g, kModeRhs, 0.0, 0, 1);
			cudaEventRecord(e1, c->stream);
			cudaEventSynchronize(e1);
			float ms = 0.f;
			cudaEventElapsedTime(&ms, e0, e1);
			if (r > 0)
				best = (r == 1 || ms < best) ? ms : best;
		}
		return best;
	};
	c->mode = 0;
	for (int g = 0; g < c->n_groups; ++g) {
		if (c->hgroups[g].n_vol == 0)
			continue;
		int bestE = c->hgroups[g].E;
		float bestT = -1.f;
		for (int E = c->gl[g].E_max; E >= 1; E /= 2) {
			c->hgroups[g].E = E;
			cudaMemcpyAsync(c->d_groups, c->hgroups.data(), c->hgroups.size() * sizeof(BGroup),
			                cudaMemcpyHostToDevice, c->stream);
			const float t = time_group(g);
			char line[128];
			snprintf(line, sizeof line, "group q=%d E=%d: %.4f ms\n", c->hgroups[g].q, E, t);
			rep += line;
			if (bestT < 0.f || t < bestT) {
				bestT = t;
				bestE = E;
			}
			if (E == 1)
				break;
		}
		c->hgroups[g].E = bestE;
	}
	BATCH_CUDA(c, cudaMemcpyAsync(c->d_groups, c->hgroups.data(), c->hgroups.size() * sizeof(BGroup),
	                              cudaMemcpyHostToDevice, c->stream));
	drop_graphs(c);
	// the three forms on RK steps (graph-replayed unless graphs are off)
	static const char* names[3] = {"plain", "fused", "branches"};
	float tmode[3] = {0.f, 0.f, 0.f};
	int best = 0;
	for (int m = 0; m < 3; ++m) {
		c->mode = m;
		if ((st = dgpu_batch_ssp_rk3_steps(c, dt, 1, nullptr)) != DGPU_OK)
			break;
		cudaEventRecord(e0, c->stream);
		if ((st = dgpu_batch_ssp_rk3_steps(c, dt, reps, nullptr)) != DGPU_OK)
			break;
		cudaEventRecord(e1, c->stream);
		cudaEventSynchronize(e1);
		cudaEventElapsedTime(&tmode[m], e0, e1);
		char line[128];
		snprintf(line, sizeof line, "%s: %.4f ms per RK3 step\n", names[m], tmode[m] / reps);
		rep += line;
		if (tmode[m] < tmode[best])
			best = m;
	}
	c->mode = best;
	cudaMemcpyAsync(coef_was ? c->u : c->ug, saved, c->ns * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
	cudaMemcpyAsync(c->rhs, saved + c->ns, c->ns * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
	cudaMemcpyAsync(c->n_corr, &n_corr0, sizeof n_corr0, cudaMemcpyHostToDevice, c->stream);
	cudaStreamSynchronize(c->stream);
	cudaFree(saved);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	c->coef_valid = coef_was;
	c->gl_valid = coef_was ? false : gl_was;
	if (report && report_len) {
		snprintf(report, report_len, "%s", rep.c_str());
	}
	return st;
}

dgpu_status dgpu_batch_set_graphs(dgpu_batch* c, int enable)
{
	if (!c || (enable != 0 && enable != 1))
		return DGPU_ERR_INVALID_ARGUMENT;
	c->use_graphs = enable != 0;
	return DGPU_OK;
}

dgpu_status dgpu_batch_get_mode(const dgpu_batch* c, int* form)
{
	if (!c || !form)
		return DGPU_ERR_INVALID_ARGUMENT;
	*form = c->mode;
	return DGPU_OK;
}

dgpu_status dgpu_batch_kernel_launches(const dgpu_batch* c, long long* n)
{
	if (!c || !n)
		return DGPU_ERR_INVALID_ARGUMENT;
	*n = c->launches;
	return DGPU_OK;
}

dgpu_status dgpu_batch_set_stream(dgpu_batch* c, void* stream)
{
	if (!c)
		return DGPU_ERR_INVALID_ARGUMENT;
	BATCH_CUDA(c, cudaStreamSynchronize(c->stream));
	if (c->own_stream)
		cudaStreamDestroy(c->stream);
	c->own_stream = false;
	c->stream = (cudaStream_t)stream;
	drop_graphs(c);
	return DGPU_OK;
}

dgpu_status dgpu_batch_positivity_corrections(dgpu_batch* c, long long* n)
{
	if (!c || !n)
		return DGPU_ERR_INVALID_ARGUMENT;
	unsigned long long v = 0;
	BATCH_CUDA(c, cudaMemcpyAsync(&v, c->n_corr, sizeof v, cudaMemcpyDeviceToHost, c->stream));
	BATCH_CUDA(c, cudaStreamSynchronize(c->stream));
	*n = (long long)v;
	return DGPU_OK;
}

}  // extern "C"
