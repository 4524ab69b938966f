// Discrete adjoint of the Navier-Stokes residual on the TP path: ubar = (dR/du)^T rbar.
//
// The forward residual (dgpu_ns.cuh), in GL nodal space with ug = V u:
//   g_v    = diag(1/(wJ)) sum_k m_k d_r_k ug                  the volume gradient (tp_ns_grad_kernel)
//   s_T, g_T = E_lf ug, E_lf g_v                              state and gradient traces
//   X, F*  = ns_face_core(s_TL, s_TR, g_TL, g_TR)             per face node
//   g      = g_v + sum_lf lift_lf(X)                          the BR2 total gradient, lift(X) = 1/(wJ) lb X on a line
//   R_gl   = diag(1/(wJ)) (sum_j Dgl_j^T fr_j(ug, g) - sum_lf E_lf^T (+-F*)),   R = V^-1 R_gl
// is transposed in reverse order:
//   xbar = diag(1/(wJ)) V^-T rbar; frbar_j = Dgl_j xbar; (ugbar, gbar) from the pointwise VJP of fr;
//   the lifting's cotangent of X per face side, lift^T gbar;                         (tp_ns_adj_volume_kernel)
//   the cotangents of both sides' state and gradient traces from the pointwise VJP of ns_face_core, with the
//   face flux's cotangent E_R xbar_R - E_L xbar_L and X's from both liftings;        (tp_ns_adj_face_kernel)
//   g_vbar = gbar + E^T g_Tbar; ugbar += E^T s_Tbar + sum_k Dgl_k^T (1/(wJ) m_k . g_vbar); ubar = V^T ugbar.
//                                                                                    (tp_ns_adj_lift_kernel)
// The pointwise VJPs run the forward flux code on dual numbers (forward mode, Dual<NV>), one block of NV inputs at a
// time, and contract the derivatives with the cotangents: the same templated code the residual and its forward-mode
// linearisation use, so the three stay consistent. The reference has no adjoint; its linearisation is checked by
// complex step (test_support_solve_dg.c:83-110), which is what the tests compare this against.
#pragma once

#include "dgpu_adjoint.cuh"
#include "dgpu_ns.cuh"

namespace dgpu {

struct NsAdjArgs {
	double* gbar;    // [v][D][NV][N]: cotangent of the BR2 total gradient at the GL nodes
	double* xbar;    // [f][side][D][NV][NF]: the liftings' cotangent of X, per face side in its own node order
	double* gtbar;   // [f][side][D][NV][NF]: cotangent of the gradient traces, per face side in its own node order
};

// (d fr / d(W, G))^T frbar at one volume node, fr = ns_flux_ref(W, G): D + 1 forward-mode passes of NV directions
// (W, then each direction's gradient components).
template <int D>
__device__ __forceinline__ void ns_flux_ref_vjp(const double* W, const double (*G)[D + 2], const double* gm,
                                                const NsPhys& ns, const double (*frb)[D + 2], double* Wb,
                                                double (*Gb)[D + 2])
{
	constexpr int NV = D + 2;
#pragma unroll 1
	for (int c = 0; c <= D; ++c) {
		Dual<NV> Wd[NV], Gd[D][NV], fr[D][NV];
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			Wd[k] = Dual<NV>(W[k]);
			if (c == 0)
				Wd[k].d[k] = 1.0;
		}
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				Gd[dir][k] = Dual<NV>(G[dir][k]);
				if (c == 1 + dir)
					Gd[dir][k].d[k] = 1.0;
			}
		ns_flux_ref<D, Dual<NV>>(Wd, Gd, gm, ns, fr);
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			double s = 0.0;
#pragma unroll
			for (int j = 0; j < D; ++j)
#pragma unroll
				for (int eq = 0; eq < NV; ++eq)
					s += frb[j][eq] * fr[j][eq].d[k];
			if (c == 0)
				Wb[k] = s;
#pragma unroll
			for (int dir = 0; dir < D; ++dir)
				if (c == 1 + dir)
					Gb[dir][k] = s;
		}
	}
}

// Per element (doubles): su (ug), st (scratch), sr (xbar), sf (D blocks: Dgl_j xbar, then 1/(wJ) gbar).
template <int D, int Q, int NV>
struct NsAdjSmem {
	static constexpr int PER_E = (3 + D) * NV * TPShape<D, Q>::N;
};

template <int D, int Q, int NV>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_ns_adj_volume_kernel(const TPOps ops, const TPParams P, const AdjArgs A, const NsAdjArgs B)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF, E = S::E, PER_E = NsAdjSmem<D, Q, NV>::PER_E;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	const int tid = threadIdx.x;
	load_ops(sops, ops);
	const int v0 = blockIdx.x * E;
	const int n_here = min(E, P.n_vol - v0);
	for (int i = tid; i < n_here * NV * N; i += blockDim.x) {
		const int e = i / (NV * N), r = i % (NV * N);
		base[e * PER_E + r] = A.u[(size_t)v0 * NV * N + i];                    // su <- u
		base[e * PER_E + 2 * NV * N + r] = A.rbar[(size_t)v0 * NV * N + i];    // sr <- rbar
	}
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	const int v = v0 + e;
	double* su = base + e * PER_E;
	double* st = su + NV * N;
	double* sr = st + NV * N;
	double* sf = sr + NV * N;

	tp_apply<D, Q, NV>(su, st, sf, sops->B, node, active);   // ug = V u
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			su[k * N + node] = st[k * N + node];
	__syncthreads();
	tp_apply<D, Q, NV>(sr, st, sf, sops->BinvT, node, active);   // xbar = diag(1/(wJ)) V^-T rbar
	const double iw = active ? P.inv_wJ[(size_t)v * N + node] : 0.0;
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			sr[k * N + node] = st[k * N + node] * iw;
	__syncthreads();
	if (active) {
		// E_lf xbar on the local faces: the face flux's cotangent is E_R xbar_R - E_L xbar_L
		for (int it = node; it < 2 * D * NF; it += N) {
			const int lf = it / NF, t = it % NF, nd = lf >> 1, side = lf & 1;
			int b0, stride;
			face_line<D, Q>(nd, t, &b0, &stride);
			const int fs = P.vol_face[(size_t)v * 2 * D + lf];
			double* adst = A.atraces + (size_t)fs * NV * NF;
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				double s = 0.0;
#pragma unroll
				for (int m = 0; m < Q; ++m)
					s += sops->lb[side][m] * sr[k * N + b0 + m * stride];
				adst[k * NF + t] = s;
			}
		}
#pragma unroll
		for (int j = 0; j < D; ++j)
			tp_pass<D, Q, NV>(sr, sf + j * NV * N, sops->Dgl, j, node);   // frbar_j = Dgl_j xbar
	}
	__syncthreads();

	double Wb[NV], Gb[D][NV];
	if (active) {
		// the total gradient as the forward volume kernel forms it: kept volume gradient + liftings of X
		double W[NV], gm[D * D], g[D][NV], frb[D][NV];
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				g[dir][k] = P.ns_gv[(((size_t)v * D + dir) * NV + k) * N + node];
				frb[dir][k] = sf[(dir * NV + k) * N + node];
			}
#pragma unroll
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int nd = lf >> 1, side = lf & 1;
			const int tf = face_node_of<D, Q>(node, nd);
			const int fs = P.vol_face[(size_t)v * 2 * D + lf], f = fs >> 1;
			const int tX = ((fs & 1) && P.nc_inv) ? P.nc_inv[(size_t)f * NF + tf] : tf;
			const double c = iw * sops->lb[side][node_coord<Q>(node, nd)];
			const double* X = P.ns_X + (size_t)f * D * NV * NF + tX;
#pragma unroll
			for (int dir = 0; dir < D; ++dir)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					g[dir][k] += c * X[(dir * NV + k) * NF];
		}
#pragma unroll
		for (int k = 0; k < NV; ++k)
			W[k] = su[k * N + node];
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			gm[c] = P.gmet[((size_t)v * D * D + c) * N + node];
		ns_flux_ref_vjp<D>(W, g, gm, P.ns, frb, Wb, Gb);
	}
	__syncthreads();   // sf is reused for 1/(wJ) gbar
	if (active) {
#pragma unroll
		for (int k = 0; k < NV; ++k)
			P.vol_gl[((size_t)v * NV + k) * N + node] = Wb[k];
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				B.gbar[(((size_t)v * D + dir) * NV + k) * N + node] = Gb[dir][k];
				sf[(dir * NV + k) * N + node] = iw * Gb[dir][k];
			}
	}
	__syncthreads();
	if (!active)
		return;
	// the liftings' cotangent of X: this volume's lifting of face node t adds 1/(wJ) lb[side][m] X(t) to the
	// gradient on the line of nodes under t
	for (int it = node; it < 2 * D * NF; it += N) {
		const int lf = it / NF, t = it % NF, nd = lf >> 1, side = lf & 1;
		int b0, stride;
		face_line<D, Q>(nd, t, &b0, &stride);
		const int fs = P.vol_face[(size_t)v * 2 * D + lf];
		double* xd = B.xbar + (size_t)fs * D * NV * NF;
		for (int c = 0; c < D * NV; ++c) {
			double s = 0.0;
#pragma unroll
			for (int m = 0; m < Q; ++m)
				s += sops->lb[side][m] * sf[c * N + b0 + m * stride];
			xd[c * NF + t] = s;
		}
	}
}

// One face node: the cotangents of both sides' state and gradient traces (each side in its own node order) from the
// pointwise VJP of ns_face_core, with the face flux's cotangent E_R xbar_R - E_L xbar_L (boundary: -E_L xbar_L) and
// X's cotangent from the liftings of both sides. Inputs in blocks of NV: W_L, G_L per direction, then (interior
// faces) W_R, G_R per direction.
template <int D, int Q, int FLUX>
__global__ void __launch_bounds__(128)
tp_ns_adj_face_kernel(const TPParams P, const AdjArgs A, const NsAdjArgs B)
{
	using S = TPShape<D, Q>;
	constexpr int NF = S::NF, NV = D + 2;
	const int gid = blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= P.n_face * NF)
		return;
	const int f = gid / NF, t = gid % NF;
	const int b = P.bnd ? P.bnd[f] : -1;
	const int tR = (b < 0 && P.nc) ? P.nc[(size_t)f * NF + t] : t;
	const double* fg = P.fgeo + (size_t)f * (D + 1) * NF;
	double n[D];
#pragma unroll
	for (int k = 0; k < D; ++k)
		n[k] = fg[k * NF + t];
	const double sc = fg[D * NF + t];
	const double lamL = P.ns_lam[(size_t)(2 * f) * NF + t];
	const double lamR = b < 0 ? P.ns_lam[(size_t)(2 * f + 1) * NF + tR] : lamL;
	const size_t oL = (size_t)(2 * f) * NV * NF, oR = (size_t)(2 * f + 1) * NV * NF;
	const size_t gL = (size_t)(2 * f) * D * NV * NF, gR = (size_t)(2 * f + 1) * D * NV * NF;
	double WL[NV], WR[NV], GtL[D][NV], GtR[D][NV], ob[NV], Xb[D][NV];
#pragma unroll
	for (int k = 0; k < NV; ++k) {
		WL[k] = P.traces[oL + k * NF + t];
		ob[k] = -A.atraces[oL + k * NF + t];
		WR[k] = 0.0;
		if (b < 0) {
			WR[k] = P.traces[oR + k * NF + tR];
			ob[k] += A.atraces[oR + k * NF + tR];
		}
	}
#pragma unroll
	for (int dir = 0; dir < D; ++dir)
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			const int c = dir * NV + k;
			GtL[dir][k] = P.ns_gtr[gL + c * NF + t];
			Xb[dir][k] = B.xbar[gL + c * NF + t];
			GtR[dir][k] = 0.0;
			if (b < 0) {
				GtR[dir][k] = P.ns_gtr[gR + c * NF + tR];
				Xb[dir][k] += B.xbar[gR + c * NF + tR];
			}
		}
	const int n_blocks = b < 0 ? 2 * (D + 1) : D + 1;
#pragma unroll 1
	for (int c = 0; c < n_blocks; ++c) {
		Dual<NV> wl[NV], wr[NV], gl[D][NV], gr[D][NV], X[D][NV], o[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			wl[k] = Dual<NV>(WL[k]);
			wr[k] = Dual<NV>(WR[k]);
			if (c == 0)
				wl[k].d[k] = 1.0;
			if (c == D + 1)
				wr[k].d[k] = 1.0;
		}
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				gl[dir][k] = Dual<NV>(GtL[dir][k]);
				gr[dir][k] = Dual<NV>(GtR[dir][k]);
				if (c == 1 + dir)
					gl[dir][k].d[k] = 1.0;
				if (c == D + 2 + dir)
					gr[dir][k].d[k] = 1.0;
			}
		ns_face_core<D, FLUX, Dual<NV>>(P, b, t, NF, n, sc, lamL, lamR, wl, wr, gl, gr, X, o);
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			double s = 0.0;
#pragma unroll
			for (int eq = 0; eq < NV; ++eq)
				s += ob[eq] * o[eq].d[k];
#pragma unroll
			for (int dir = 0; dir < D; ++dir)
#pragma unroll
				for (int eq = 0; eq < NV; ++eq)
					s += Xb[dir][eq] * X[dir][eq].d[k];
			if (c == 0)
				A.wbar[oL + k * NF + t] = s;
			else if (c <= D)
				B.gtbar[gL + ((c - 1) * NV + k) * NF + t] = s;
			else if (c == D + 1)
				A.wbar[oR + k * NF + tR] = s;
			else
				B.gtbar[gR + ((c - D - 2) * NV + k) * NF + tR] = s;
		}
	}
}

// g_vbar = gbar + E^T g_Tbar; ugbar = (volume part) + E^T s_Tbar + sum_k Dgl_k^T (1/(wJ) sum_dir m(k, dir) g_vbar[dir]);
// ubar = V^T ugbar. Per element (doubles): h (D blocks), sa, sb, sc.
template <int D, int Q, int NV>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_ns_adj_lift_kernel(const TPOps ops, const TPParams P, const AdjArgs A, const NsAdjArgs B)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF, E = S::E, PER_E = NsAdjSmem<D, Q, NV>::PER_E;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	const int tid = threadIdx.x;
	load_ops(sops, ops);
	const int v0 = blockIdx.x * E;
	const int n_here = min(E, P.n_vol - v0);
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	const int v = v0 + e;
	double* h = base + e * PER_E;
	double* sa = h + D * NV * N;
	double* sb = sa + NV * N;
	double* sc = sb + NV * N;
	double ub[NV];
	if (active) {
		double gv[D][NV];
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				gv[dir][k] = B.gbar[(((size_t)v * D + dir) * NV + k) * N + node];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			ub[k] = P.vol_gl[((size_t)v * NV + k) * N + node];
#pragma unroll
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int fs = P.vol_face[(size_t)v * 2 * D + lf];
			const int nd = lf >> 1;
			const int t = face_node_of<D, Q>(node, nd);
			const double l = sops->lb[lf & 1][node_coord<Q>(node, nd)];
			const double* ws = A.wbar + (size_t)fs * NV * NF;        // this side's own node order
			const double* gs = B.gtbar + (size_t)fs * D * NV * NF;
#pragma unroll
			for (int k = 0; k < NV; ++k)
				ub[k] += l * ws[k * NF + t];
#pragma unroll
			for (int dir = 0; dir < D; ++dir)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					gv[dir][k] += l * gs[(dir * NV + k) * NF + t];
		}
		const double iw = P.inv_wJ[(size_t)v * N + node];
		double gm[D * D];
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			gm[c] = P.gmet[((size_t)v * D * D + c) * N + node];
		// cotangent of the collocation derivative d_r_k ug: 1/(wJ) sum_dir m(k, dir) g_vbar[dir]
#pragma unroll
		for (int kk = 0; kk < D; ++kk)
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				double s = 0.0;
#pragma unroll
				for (int dir = 0; dir < D; ++dir)
					s += gm[kk * D + dir] * gv[dir][k];
				h[(kk * NV + k) * N + node] = iw * s;
			}
	}
	__syncthreads();
	if (active) {
#pragma unroll
		for (int kk = 0; kk < D; ++kk) {
			const int stride = (kk == 0 ? 1 : (kk == 1 ? Q : Q * Q));
			const int a = node_coord<Q>(node, kk);
			const int b0 = node - a * stride;
#pragma unroll
			for (int m = 0; m < Q; ++m) {
				const double w = sops->Dgl[m][a];
#pragma unroll
				for (int k = 0; k < NV; ++k)
					ub[k] += w * h[(kk * NV + k) * N + b0 + m * stride];
			}
		}
#pragma unroll
		for (int k = 0; k < NV; ++k)
			sa[k * N + node] = ub[k];
	}
	__syncthreads();
	tp_apply<D, Q, NV>(sa, sb, sc, sops->BT, node, active);   // ubar = V^T ugbar
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			A.ubar[((size_t)v * NV + k) * N + node] = sb[k * N + node];
}

}  // namespace dgpu
