// Navier-Stokes (BR2) in the batched mixed-order context: QUAD/HEX groups of any p = 1..4, faces at
// p_f = max(p_L, p_R) (face_solver.c:123-132).
//
// The uniform path's GL-space reduction of the reference's BR2 operators (compute_grad_coef_dg_T.c:60-316,
// constructor_partial_grad_fc_interp, compute_face_rlhs_dg_T.c:239-295; see dgpu_ns.cuh) carries over with the
// tangential interpolation I (the element's GL(q) points -> the face's GL(q_f) points) between a volume and a face
// of a higher order:
//   lifting of X into the volume's GL values:      diag(1/(w J)) E^T I^T X,
//   the face's own lifting at the face nodes:       I diag(lambda) I^T X,   lambda(t) = sum_m lb[m]^2 / (w J)(t, m),
// X = w_f J_f n (s_R - s_L) / 2 at the face's q_f nodes. With q_f = q, I is the identity and both reduce to the
// uniform kernels' forms. Per stage:
//   bns_grad   (per group)       GL state, the physical volume gradient (kept), state and gradient traces at q_f;
//   bns_jump   (per face node)   w_f J_f (W_R - W_L) / 2 (W_R the boundary value on a boundary face);
//   bns_volume (per group)       I^T X of every face: the total gradient (kept + liftings) for the Euler and
//                                viscous contravariant flux and its Dgl^T contraction, and I diag(lambda) I^T X of
//                                each face side for the face kernel;
//   bns_face   (per face node)   partial face gradients g_tr + eta I diag(lambda) I^T X, numerical + central
//                                viscous flux (ns_face_flux);
// then the batched lift of dgpu_batched.cuh, as for Euler.
#pragma once

#include "dgpu_batched.cuh"
#include "dgpu_ns.cuh"

namespace dgpu {

// Shared memory per element (doubles) of the two element bodies.
template <int D, int Q, int NV>
struct BnsSmem {
	static constexpr int N = TPShape<D, Q>::N;
	static constexpr int NFQ = TPShape<D, Q>::NF;
	static constexpr int NF_MAX = (D == 2 ? kQMax : kQMax * kQMax);                // nodes of a face at q_f = 5
	static constexpr int GRAD = (1 + D) * NV * N + 2 * D * (1 + D) * NV * NFQ;   // su, sd, traces of both
	// su, sf, I^T X per face, X of one face at its q_f nodes
	static constexpr int VOL = (1 + D) * NV * N + 2 * D * D * NV * NFQ + D * NV * NF_MAX;
	static constexpr int MAX = GRAD > VOL ? GRAD : VOL;
};

// C components at the element's own points of one local face (src [C][NFQ]) written at the face's q_f points
// (dst [C][nff]): a copy when q_f == Q, else the tangential GL(Q) -> GL(q_f) interpolation (separable in 3D).
// The element's threads (node = 0 .. N-1) share the work.
template <int D, int Q>
__device__ __forceinline__ void bface_put(const BatchOps* sops, int qf, int C, const double* src, double* dst,
                                          int node)
{
	constexpr int N = TPShape<D, Q>::N, NFQ = TPShape<D, Q>::NF;
	if (qf == Q) {
		for (int it = node; it < C * NFQ; it += N)
			dst[it] = src[it];
		return;
	}
	const double(*I)[kQMax] = sops->Iup[qf];
	if (D == 2) {
		for (int it = node; it < C * qf; it += N) {
			const int k = it / qf, i = it % qf;
			double s = 0.0;
#pragma unroll
			for (int a = 0; a < Q; ++a)
				s += I[i][a] * src[k * NFQ + a];
			dst[k * qf + i] = s;
		}
	} else {
		const int nff = qf * qf;
		for (int it = node; it < C * qf; it += N) {
			const int k = it / qf, i0 = it % qf;
			double r[Q];
#pragma unroll
			for (int b = 0; b < Q; ++b) {
				double acc = 0.0;
#pragma unroll
				for (int a = 0; a < Q; ++a)
					acc += I[i0][a] * src[k * NFQ + a + Q * b];
				r[b] = acc;
			}
			for (int i1 = 0; i1 < qf; ++i1) {
				double s = 0.0;
#pragma unroll
				for (int b = 0; b < Q; ++b)
					s += I[i1][b] * r[b];
				dst[k * nff + i0 + qf * i1] = s;
			}
		}
	}
}

// The transpose: C components given at the face's q_f points by src(c, i) (i in the element's own face-node
// order), summed onto the element's own points (out [C][NFQ]).
template <int D, int Q, typename F>
__device__ __forceinline__ void bface_get(const BatchOps* sops, int qf, int C, F src, double* out, int node)
{
	constexpr int N = TPShape<D, Q>::N, NFQ = TPShape<D, Q>::NF;
	if (qf == Q) {
		for (int it = node; it < C * NFQ; it += N)
			out[it] = src(it / NFQ, it % NFQ);
		return;
	}
	const double(*I)[kQMax] = sops->Iup[qf];
	if (D == 2) {
		for (int it = node; it < C * Q; it += N) {
			const int k = it / Q, t = it % Q;
			double s = 0.0;
			for (int i = 0; i < qf; ++i)
				s += I[i][t] * src(k, i);
			out[k * NFQ + t] = s;
		}
	} else {
		for (int it = node; it < C * Q; it += N) {
			const int k = it / Q, a = it % Q;
			double r[kQMax];
#pragma unroll
			for (int i1 = 0; i1 < kQMax; ++i1) {
				double acc = 0.0;
				if (i1 < qf)
					for (int i0 = 0; i0 < qf; ++i0)
						acc += I[i0][a] * src(k, i0 + qf * i1);
				r[i1] = acc;
			}
#pragma unroll
			for (int bb = 0; bb < Q; ++bb) {
				double s = 0.0;
#pragma unroll
				for (int i1 = 0; i1 < kQMax; ++i1)
					if (i1 < qf)
						s += I[i1][bb] * r[i1];
				out[k * NFQ + a + Q * bb] = s;
			}
		}
	}
}

// Start index and stride of the line of volume nodes under own face point t of local face lf.
template <int D, int Q>
__device__ __forceinline__ void bface_line(int lf, int t, int* base, int* stride)
{
	face_line<D, Q>(lf >> 1, t, base, stride);
}

// ---- gradient, kept, and the traces of state and gradient at each face's order ----
template <int D, int Q, int NV, bool GLL_IN>
__device__ void bns_grad_body(const BParams& P, const BatchOps* sops, const BGroup& G, int e0, int E,
                              const double* __restrict__ u, double* base)
{
	constexpr int N = TPShape<D, Q>::N, NFQ = TPShape<D, Q>::NF, C = (1 + D) * NV;
	constexpr int PER_E = BnsSmem<D, Q, NV>::MAX;
	const int tid = threadIdx.x, n_here = min(E, G.n_vol - e0);
	const double* ublk = u + G.state_off + (long long)e0 * NV * N;
	for (int i = tid; i < n_here * NV * N; i += blockDim.x)
		base[(i / (NV * N)) * PER_E + i % (NV * N)] = ublk[i];
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* su = base + e * PER_E;
	double* sd = su + NV * N;          // D NV N: derivatives, then the physical gradient
	double* str = sd + D * NV * N;     // [lf][C][NFQ]: state (NV) and gradient (D NV) traces at own points
	if (GLL_IN) {
		tp_apply<D, Q, NV>(su, sd, sd + NV * N, sops->t.B, node, active);
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				su[k * N + node] = sd[k * N + node];
		__syncthreads();
	}
	if (active)
#pragma unroll
		for (int k = 0; k < D; ++k)
			tp_pass<D, Q, NV>(su, sd + k * NV * N, sops->t.Dgl, k, node);
	__syncthreads();
	double g[D][NV];
	const long long el = (long long)(e0 + e);
	if (active) {
		const double iwJ = P.inv_wJ[G.wj_off + el * N + node];
		const double* gmp = P.gmet + G.gmet_off + el * D * D * N;
		double gm[D * D];
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			gm[c] = gmp[c * N + node];
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int var = 0; var < NV; ++var) {
				double a = 0.0;
#pragma unroll
				for (int k = 0; k < D; ++k)
					a += gm[k * D + dir] * sd[(k * NV + var) * N + node];   // w J dr_k/dx_dir d_r_k u
				g[dir][var] = iwJ * a;
			}
	}
	__syncthreads();
	if (active) {
		double* gv = P.ns_gv + (long long)D * G.state_off + el * D * NV * N;
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int var = 0; var < NV; ++var) {
				sd[(dir * NV + var) * N + node] = g[dir][var];
				gv[(dir * NV + var) * N + node] = g[dir][var];
			}
	}
	__syncthreads();
	if (active) {
		for (int it = node; it < 2 * D * NFQ; it += N) {
			const int lf = it / NFQ, t = it % NFQ, side = lf & 1;
			int b, stride;
			bface_line<D, Q>(lf, t, &b, &stride);
			for (int c = 0; c < C; ++c) {
				const double* src = c < NV ? su + c * N : sd + (c - NV) * N;
				double s = 0.0;
#pragma unroll
				for (int m = 0; m < Q; ++m)
					s += sops->t.lb[side][m] * src[b + m * stride];
				str[(lf * C + c) * NFQ + t] = s;
			}
		}
	}
	__syncthreads();
	if (active) {
		const int4* ef = P.elf + (G.elem0 + el) * kMaxLf;
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int4 fd = ef[lf];
			const int qf = fd.z, nff = (D == 2 ? qf : qf * qf);
			const long long fb = P.fbase[fd.x];
			bface_put<D, Q>(sops, qf, NV, str + lf * C * NFQ, P.traces + 2 * NV * fb + (long long)fd.y * NV * nff,
			                node);
			bface_put<D, Q>(sops, qf, D * NV, str + (lf * C + NV) * NFQ,
			                P.ns_gtr + 2 * D * NV * fb + (long long)fd.y * D * NV * nff, node);
		}
	}
	__syncthreads();   // shared memory is reused by the next tile
}

// ---- the jump w_f J_f (W_R - W_L) / 2 at a face node (side-0 node order) ----
template <int D, int NV>
__device__ __forceinline__ void bns_jump_node(const BParams& P, int f, int i, int nff)
{
	const long long fb = P.fbase[f];
	const double* tL = P.traces + 2 * NV * fb;
	const double* fg = P.fgeo + (D + 1) * fb;
	double WL[NV], WR[NV], n[D];
#pragma unroll
	for (int k = 0; k < NV; ++k)
		WL[k] = tL[k * nff + i];
#pragma unroll
	for (int k = 0; k < D; ++k)
		n[k] = fg[k * nff + i];
	const int code = P.fbc ? P.fbc[f] : -1;
	if (code < 0) {
		const int iR = P.nc ? P.nc[fb + i] : i;
#pragma unroll
		for (int k = 0; k < NV; ++k)
			WR[k] = tL[NV * nff + k * nff + iR];
	} else {
		ns_boundary_state<D, double>(code, WL, P.fext + NV * fb + i, nff, n, P.bc_data, WR);
	}
	const double h = 0.5 * fg[D * nff + i];
#pragma unroll
	for (int k = 0; k < NV; ++k)
		P.ns_dw[NV * fb + k * nff + i] = h * (WR[k] - WL[k]);
}

// ---- liftings, the total gradient, the Euler and viscous flux and its contraction; each face side's I lambda I^T X
template <int D, int Q, int NV, bool GLL_IN>
__device__ void bns_volume_body(const BParams& P, const BatchOps* sops, const BGroup& G, int e0, int E,
                                const double* __restrict__ u, double* base)
{
	constexpr int N = TPShape<D, Q>::N, NFQ = TPShape<D, Q>::NF, C = D * NV;
	constexpr int PER_E = BnsSmem<D, Q, NV>::MAX;
	const int tid = threadIdx.x, n_here = min(E, G.n_vol - e0);
	const double* ublk = u + G.state_off + (long long)e0 * NV * N;
	for (int i = tid; i < n_here * NV * N; i += blockDim.x)
		base[(i / (NV * N)) * PER_E + i % (NV * N)] = ublk[i];
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* su = base + e * PER_E;
	double* sf = su + NV * N;          // D NV N: contravariant flux (the GLL -> GL temporaries first)
	double* sx = sf + D * NV * N;      // [lf][C][NFQ]: I^T X at the element's own face points
	double* sxf = sx + 2 * D * C * NFQ;   // [C][nff]: X of one face at its q_f nodes, in this side's node order
	if (GLL_IN) {
		tp_apply<D, Q, NV>(su, sf, sf + NV * N, sops->t.B, node, active);
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				su[k * N + node] = sf[k * N + node];
		__syncthreads();
	}
	const long long el = (long long)(e0 + e);
	const int4* ef = P.elf + (G.elem0 + (active ? el : 0)) * kMaxLf;
	for (int lf = 0; lf < 2 * D; ++lf) {   // every thread of the CTA: the loop synchronises
		int qf = Q, nff = 0;
		if (active) {
			const int4 fd = ef[lf];
			qf = fd.z;
			nff = (D == 2 ? qf : qf * qf);
			const long long fb = P.fbase[fd.x];
			// side 1 reads the side-0-ordered jump and normal at its own nodes through the inverse permutation;
			// X = n (side 0's) times the jump serves both sides (the same values seen from either side). Each
			// value is read from global memory once, into sxf.
			const int* ci = (fd.y == 1 && P.nc_inv) ? P.nc_inv + fb : nullptr;
			const double* dw = P.ns_dw + NV * fb;
			const double* fg = P.fgeo + (D + 1) * fb;
			for (int i = node; i < nff; i += N) {
				const int j = ci ? ci[i] : i;
				double w[NV];
#pragma unroll
				for (int k = 0; k < NV; ++k)
					w[k] = dw[k * nff + j];
#pragma unroll
				for (int dir = 0; dir < D; ++dir) {
					const double nd = fg[dir * nff + j];
#pragma unroll
					for (int k = 0; k < NV; ++k)
						sxf[(dir * NV + k) * nff + i] = nd * w[k];
				}
			}
		}
		__syncthreads();
		if (active) {
			auto src = [&](int c, int i) { return sxf[c * nff + i]; };
			bface_get<D, Q>(sops, qf, C, src, sx + lf * C * NFQ, node);
		}
		__syncthreads();
	}
	double fr[D][NV];
	const double* iwJp = P.inv_wJ + G.wj_off + el * N;
	if (active) {
		double g[D][NV];
		const double* gv = P.ns_gv + (long long)D * G.state_off + el * D * NV * N;
		const double iwJ = iwJp[node];
#pragma unroll
		for (int c = 0; c < C; ++c)
			g[c / NV][c % NV] = gv[c * N + node];
#pragma unroll
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int nd = lf >> 1;
			const double l = iwJ * sops->t.lb[lf & 1][node_coord<Q>(node, nd)];
			const double* x = sx + lf * C * NFQ + face_node_of<D, Q>(node, nd);
#pragma unroll
			for (int c = 0; c < C; ++c)
				g[c / NV][c % NV] += l * x[c * NFQ];
		}
		double W[NV], gm[D * D];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			W[k] = su[k * N + node];
		const double* gmp = P.gmet + G.gmet_off + el * D * D * N;
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			gm[c] = gmp[c * N + node];
		ns_flux_ref<D, double>(W, g, gm, P.ns, fr);
	}
	__syncthreads();   // every thread is done with sx as I^T X, and with sf as temporaries
	if (active) {
#pragma unroll
		for (int j = 0; j < D; ++j)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				sf[(j * NV + k) * N + node] = fr[j][k];
		// lambda I^T X at the own face points
		for (int it = node; it < 2 * D * NFQ; it += N) {
			const int lf = it / NFQ, t = it % NFQ, side = lf & 1;
			int b, stride;
			bface_line<D, Q>(lf, t, &b, &stride);
			double lam = 0.0;
#pragma unroll
			for (int m = 0; m < Q; ++m) {
				const double l = sops->t.lb[side][m];
				lam += l * l * iwJp[b + m * stride];
			}
			for (int c = 0; c < C; ++c)
				sx[(lf * C + c) * NFQ + t] *= lam;
		}
	}
	__syncthreads();
	if (active) {
		double acc[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			acc[k] = 0.0;
#pragma unroll
		for (int j = 0; j < D; ++j) {
			const int stride = (j == 0 ? 1 : (j == 1 ? Q : Q * Q));
			const int a = node_coord<Q>(node, j);
			const int b0 = node - a * stride;
#pragma unroll
			for (int m = 0; m < Q; ++m) {
				const double w = sops->t.Dgl[m][a];
#pragma unroll
				for (int k = 0; k < NV; ++k)
					acc[k] += w * sf[(j * NV + k) * N + b0 + m * stride];
			}
		}
		double* vg = P.vol_gl + G.state_off + el * NV * N;
#pragma unroll
		for (int k = 0; k < NV; ++k)
			vg[k * N + node] = acc[k];
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int4 fd = ef[lf];
			const int qf = fd.z, nff = (D == 2 ? qf : qf * qf);
			bface_put<D, Q>(sops, qf, C, sx + lf * C * NFQ,
			                P.ns_y + 2 * D * NV * P.fbase[fd.x] + (long long)fd.y * D * NV * nff, node);
		}
	}
	__syncthreads();   // shared memory is reused by the next tile
}

// ---- the face flux at a face node ----
template <int D, int NV, int FLUX>
__device__ __forceinline__ void bns_face_node(const BParams& P, int f, int i, int nff)
{
	const long long fb = P.fbase[f];
	const double* tL = P.traces + 2 * NV * fb;
	const double* fg = P.fgeo + (D + 1) * fb;
	const double* gtr = P.ns_gtr + 2 * D * NV * fb;
	const double* y = P.ns_y + 2 * D * NV * fb;
	double WL[NV], WR[NV], n[D], GL[D][NV], GR[D][NV];
#pragma unroll
	for (int k = 0; k < NV; ++k)
		WL[k] = tL[k * nff + i];
#pragma unroll
	for (int k = 0; k < D; ++k)
		n[k] = fg[k * nff + i];
	const int code = P.fbc ? P.fbc[f] : -1;
	const int iR = (code < 0 && P.nc) ? P.nc[fb + i] : i;
#pragma unroll
	for (int c = 0; c < D * NV; ++c)
		GL[c / NV][c % NV] = gtr[c * nff + i] + P.ns_eta * y[c * nff + i];
	if (code < 0) {
#pragma unroll
		for (int k = 0; k < NV; ++k)
			WR[k] = tL[NV * nff + k * nff + iR];
#pragma unroll
		for (int c = 0; c < D * NV; ++c)
			GR[c / NV][c % NV] = gtr[(D * NV + c) * nff + iR] + P.ns_eta * y[(D * NV + c) * nff + iR];
	}
	double X[D][NV], o[NV];
	const double* ext = code >= 0 ? P.fext + NV * fb + i : nullptr;
	ns_face_flux<D, FLUX, double>(code, ext, nff, P.bc_data, P.ns, 0.0, n, fg[D * nff + i], 0.0, 0.0, WL, WR, GL,
	                              GR, X, o);
#pragma unroll
	for (int k = 0; k < NV; ++k)
		P.nnf[NV * fb + k * nff + i] = o[k];
}

// ---- kernels ----
template <int D, int Q, int NV, bool GLL_IN>
__global__ void __launch_bounds__(256) bns_grad_group_kernel(const BParams P, int g, const double* __restrict__ u)
{
	extern __shared__ double smem[];
	BatchOps* sops = reinterpret_cast<BatchOps*>(smem);
	const BGroup G = P.groups[g];
	load_batch_ops(sops, &P.ops[g]);
	__syncthreads();
	bns_grad_body<D, Q, NV, GLL_IN>(P, sops, G, blockIdx.x * G.E_ns, G.E_ns, u, smem + sizeof(BatchOps) / 8);
}

template <int D, int Q, int NV, bool GLL_IN>
__global__ void __launch_bounds__(256) bns_volume_group_kernel(const BParams P, int g, const double* __restrict__ u)
{
	extern __shared__ double smem[];
	BatchOps* sops = reinterpret_cast<BatchOps*>(smem);
	const BGroup G = P.groups[g];
	load_batch_ops(sops, &P.ops[g]);
	if (blockIdx.x == 0 && threadIdx.x == 0 && P.max_bits && G.elem0 == 0)   // first non-empty group
		*P.max_bits = 0ull;
	__syncthreads();
	bns_volume_body<D, Q, NV, GLL_IN>(P, sops, G, blockIdx.x * G.E_ns, G.E_ns, u, smem + sizeof(BatchOps) / 8);
}

template <int D, int NV>
__global__ void __launch_bounds__(256) bns_jump_kernel(const BParams P, const int* __restrict__ node_face,
                                                       long long n_nodes)
{
	for (long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x; gid < n_nodes;
	     gid += (long long)gridDim.x * blockDim.x) {
		const int f = node_face[gid];
		const long long fb = P.fbase[f];
		bns_jump_node<D, NV>(P, f, (int)(gid - fb), (int)(P.fbase[f + 1] - fb));
	}
}

template <int D, int NV, int FLUX>
__global__ void __launch_bounds__(128) bns_face_kernel(const BParams P, const int* __restrict__ node_face,
                                                       long long n_nodes)
{
	for (long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x; gid < n_nodes;
	     gid += (long long)gridDim.x * blockDim.x) {
		const int f = node_face[gid];
		const long long fb = P.fbase[f];
		bns_face_node<D, NV, FLUX>(P, f, (int)(gid - fb), (int)(P.fbase[f + 1] - fb));
	}
}

}  // namespace dgpu
