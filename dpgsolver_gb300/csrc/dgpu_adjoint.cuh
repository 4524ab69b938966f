// Discrete adjoint of the explicit DG residual: the vector-Jacobian product  ubar = (dR/du)^T rbar.
//
// With ug = V u, X = sum_j Dgl_j^T fr_j(ug) - sum_lf E_lf^T S_f F*(traces), R = V^-1 diag(1/(wJ)) X (the factored
// form of dgpu_tp.cuh), the transpose is applied in reverse order:
//   xbar  = diag(1/(wJ)) V^-T rbar                              (GL space)
//   ubar_g = sum_j (dfr_j/dU)^T (Dgl_j xbar)                    (volume, pointwise Jacobians by reverse mode)
//          + sum_lf E_lf^T (dF*/dW_side)^T S_f (E_R xbar_R - E_L xbar_L)   (faces)
//   ubar  = V^T ubar_g
// Kernels: tp_adj_volume_kernel (V u, forward traces, xbar, adjoint traces, volume part), tp_adj_face_kernel
// (numerical-flux Jacobians by forward-mode dual numbers, per side), tp_adj_lift_kernel (face part and V^T).
// The reference has no adjoint; its linearisation is checked by complex step (test_support_solve_dg.c:83-110),
// which is what the tests compare this against.
#pragma once

#include "dgpu_tp.cuh"

namespace dgpu {

struct AdjArgs {
	const double* u;      // state (GLL coefficients) at which the Jacobian is taken
	const double* rbar;   // cotangent of R (GLL layout)
	double* ubar;         // result (GLL layout)
	double* atraces;      // [f][2][NV][NF]: E_lf xbar of each side
	double* wbar;         // [f][2][NV][NF]: (dF*/dW_side)^T S_f Fbar, in each side's own face-node order
};

// Reverse mode of euler_flux_ref: adds (dfr/dW)^T sbar to Wbar, sbar[j][eq] the cotangent of fr[j][eq].
template <int D>
__device__ __forceinline__ void euler_flux_ref_vjp(const double* W, const double* g, const double (*sbar)[D + 2],
                                                   double* Wbar)
{
	const double rho = W[0], E = W[D + 1];
	const double rho_inv = 1.0 / rho;
	double u[D], U[D];
	double V2 = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k) {
		u[k] = rho_inv * W[1 + k];
		V2 += u[k] * u[k];
	}
	const double p = kGm1 * (E - 0.5 * rho * V2);
	const double Ep = E + p;
	double rhob = 0.0, Eb = 0.0, pb = 0.0;
	double mb[D], ub[D];
#pragma unroll
	for (int k = 0; k < D; ++k) {
		mb[k] = 0.0;
		ub[k] = 0.0;
	}
#pragma unroll
	for (int j = 0; j < D; ++j) {
		U[j] = 0.0;
#pragma unroll
		for (int i = 0; i < D; ++i)
			U[j] += g[j * D + i] * u[i];
		// fr_j[0] = rho U_j ; fr_j[1+m] = m_m U_j + p g_jm ; fr_j[D+1] = (E+p) U_j
		double Ub = sbar[j][0] * rho + sbar[j][D + 1] * Ep;
		rhob += sbar[j][0] * U[j];
#pragma unroll
		for (int m = 0; m < D; ++m) {
			Ub += sbar[j][1 + m] * W[1 + m];
			mb[m] += sbar[j][1 + m] * U[j];
			pb += sbar[j][1 + m] * g[j * D + m];
		}
		Eb += sbar[j][D + 1] * U[j];
		pb += sbar[j][D + 1] * U[j];
		// U_j = sum_i g_ji u_i
#pragma unroll
		for (int i = 0; i < D; ++i)
			ub[i] += Ub * g[j * D + i];
	}
	// p = GM1 (E - 0.5 rho V2)
	Eb += kGm1 * pb;
	rhob += -0.5 * kGm1 * V2 * pb;
	const double V2b = -0.5 * kGm1 * rho * pb;
	double rinvb = 0.0;
#pragma unroll
	for (int i = 0; i < D; ++i) {
		ub[i] += 2.0 * u[i] * V2b;          // V2 = sum u_i^2
		mb[i] += ub[i] * rho_inv;           // u_i = m_i rho_inv
		rinvb += ub[i] * W[1 + i];
	}
	rhob += -rinvb * rho_inv * rho_inv;   // rho_inv = 1 / rho
	Wbar[0] += rhob;
#pragma unroll
	for (int i = 0; i < D; ++i)
		Wbar[1 + i] += mb[i];
	Wbar[D + 1] += Eb;
}

// (dF*/dW_side)^T Fbar for one face node, side = 0 (left) or 1 (right), by forward-mode duals in NV directions.
template <int D, int NV, int FLUX>
__device__ __forceinline__ void num_flux_vjp_side(const double* WL, const double* WR, const double* n,
                                                  const double* Fbar, int side, double* Wbar)
{
	Dual<NV> L[NV], R[NV], F[NV];
#pragma unroll
	for (int k = 0; k < NV; ++k) {
		L[k] = Dual<NV>(WL[k]);
		R[k] = Dual<NV>(WR[k]);
	}
	if (side == 0) {
#pragma unroll
		for (int k = 0; k < NV; ++k)
			L[k].d[k] = 1.0;
	} else {
#pragma unroll
		for (int k = 0; k < NV; ++k)
			R[k].d[k] = 1.0;
	}
	if constexpr (FLUX == kRoePike)
		num_flux_roe_pike<D, Dual<NV>>(L, R, n, F);
	else
		num_flux_lax_friedrichs<D, Dual<NV>>(L, R, n, F);
#pragma unroll
	for (int k = 0; k < NV; ++k) {
		double s = 0.0;
#pragma unroll
		for (int eq = 0; eq < NV; ++eq)
			s += Fbar[eq] * F[eq].d[k];
		Wbar[k] = s;
	}
}

// (d/dW_L F*(W_L, W_b(W_L)))^T Fbar at a boundary face node, W_b the boundary value of its BC (the exterior state
// is data and carries no derivative).
template <int D, int NV, int FLUX>
__device__ __forceinline__ void num_flux_vjp_boundary(const TPParams& P, int b, int i, int NF, const double* WL,
                                                      const double* n, const double* Fbar, double* Wbar)
{
	Dual<NV> L[NV], R[NV], F[NV];
#pragma unroll
	for (int k = 0; k < NV; ++k) {
		L[k] = Dual<NV>(WL[k]);
		L[k].d[k] = 1.0;
	}
	boundary_value<D, NV, kEuler, Dual<NV>>(P, b, i, NF, L, n, R);
	if constexpr (FLUX == kRoePike)
		num_flux_roe_pike<D, Dual<NV>>(L, R, n, F);
	else
		num_flux_lax_friedrichs<D, Dual<NV>>(L, R, n, F);
#pragma unroll
	for (int k = 0; k < NV; ++k) {
		double s = 0.0;
#pragma unroll
		for (int eq = 0; eq < NV; ++eq)
			s += Fbar[eq] * F[eq].d[k];
		Wbar[k] = s;
	}
}

// ---------------------------------------------------------------------------------------------------------------
template <int D, int Q, int NV, int PDE>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_adj_volume_kernel(const TPOps ops, const TPParams P, const AdjArgs A)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF, E = S::E;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	// per element: su (ug), st (tmp), sr (xbar), sf (D blocks: Dgl_j xbar)
	constexpr int PER_E = NV * N * 3 + D * NV * N;

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

	// ug = V u (into st, then su)
	tp_apply<D, Q, NV>(su, st, sf, sops->B, node, active);
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			su[k * N + node] = st[k * N + node];
	__syncthreads();
	// xbar = diag(1/(wJ)) V^-T rbar (into st, scaled into sr)
	tp_apply<D, Q, NV>(sr, st, sf, sops->BinvT, node, active);
	if (active) {
		const double iw = P.inv_wJ[(size_t)v * N + node];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			sr[k * N + node] = st[k * N + node] * iw;
	}
	__syncthreads();

	if (active) {
		// forward traces of ug and adjoint traces of xbar on the 2D local faces
		for (int it = node; it < 2 * D * NF; it += N) {
			const int lf = it / NF, t = it % NF;
			const int nd = lf >> 1, side = lf & 1;
			int t0, t1;
			if (D == 2) {
				t0 = t; t1 = 0;
			} else {
				t0 = t % Q; t1 = t / Q;
			}
			int stride_n, base_n;
			if (D == 2) {
				stride_n = (nd == 0 ? 1 : Q);
				base_n = (nd == 0 ? t0 * Q : t0);
			} else {
				stride_n = (nd == 0 ? 1 : (nd == 1 ? Q : Q * Q));
				base_n = (nd == 0 ? t0 * Q + t1 * Q * Q : (nd == 1 ? t0 + t1 * Q * Q : t0 + t1 * Q));
			}
			const int fs = P.vol_face[(size_t)v * 2 * D + lf];
			double* dst = P.traces + (size_t)fs * NV * NF;
			double* adst = A.atraces + (size_t)fs * NV * NF;
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				double s = 0.0, sa = 0.0;
#pragma unroll
				for (int m = 0; m < Q; ++m) {
					s += sops->lb[side][m] * su[k * N + base_n + m * stride_n];
					sa += sops->lb[side][m] * sr[k * N + base_n + m * stride_n];
				}
				dst[k * NF + t] = s;
				adst[k * NF + t] = sa;
			}
		}
		// Dgl_j xbar for each direction j
#pragma unroll
		for (int j = 0; j < D; ++j)
			tp_pass<D, Q, NV>(sr, sf + j * NV * N, sops->Dgl, j, node);
	}
	__syncthreads();

	if (active) {
		double W[NV], Wb[NV], g[D * D];
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			W[k] = su[k * N + node];
			Wb[k] = 0.0;
		}
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			g[c] = P.gmet[((size_t)v * D * D + c) * N + node];
		if constexpr (PDE == kEuler) {
			double sb[D][D + 2];
#pragma unroll
			for (int j = 0; j < D; ++j)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					sb[j][k] = sf[(j * NV + k) * N + node];
			euler_flux_ref_vjp<D>(W, g, sb, Wb);
		} else {
#pragma unroll
			for (int j = 0; j < D; ++j) {
				double gb = 0.0;
#pragma unroll
				for (int i = 0; i < D; ++i)
					gb += g[j * D + i] * P.b_adv[i];
				Wb[0] += gb * sf[j * N + node];
			}
		}
#pragma unroll
		for (int k = 0; k < NV; ++k)
			P.vol_gl[((size_t)v * NV + k) * N + node] = Wb[k];
	}
}

template <int D, int Q, int NV, int PDE, int FLUX>
__global__ void __launch_bounds__(128)
tp_adj_face_kernel(const TPParams P, const AdjArgs A)
{
	using S = TPShape<D, Q>;
	constexpr int NF = S::NF;
	const int gid = blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= P.n_face * NF)
		return;
	const int f = gid / NF, i = gid % NF;
	const int b = P.bnd ? P.bnd[f] : -1;
	const double* tL = P.traces + (size_t)(2 * f) * NV * NF;
	const double* aL = A.atraces + (size_t)(2 * f) * NV * NF;
	const double* fg = P.fgeo + (size_t)f * (D + 1) * NF;
	double WL[NV], WR[NV], Fb[NV], n[D];
	const double sc = fg[D * NF + i];
#pragma unroll
	for (int k = 0; k < D; ++k)
		n[k] = fg[k * NF + i];
	double* wL = A.wbar + (size_t)(2 * f) * NV * NF;
	if (b >= 0) {
		// boundary face: R_L -= E_L^T S F*(W_L, W_b(W_L)) only, so Fbar = -S E_L xbar_L
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			WL[k] = tL[k * NF + i];
			Fb[k] = -sc * aL[k * NF + i];
		}
		if constexpr (PDE == kEuler) {
			double WbL[NV];
			num_flux_vjp_boundary<D, NV, FLUX>(P, b, i, NF, WL, n, Fb, WbL);
#pragma unroll
			for (int k = 0; k < NV; ++k)
				wL[k * NF + i] = WbL[k];
		} else {
			double b_dot_n = 0.0;
#pragma unroll
			for (int k = 0; k < D; ++k)
				b_dot_n += P.b_adv[k] * n[k];
			// outflow (b.n > 0): the flux is b.n u_L on either branch of the upwind flux; inflow: the exterior
			wL[i] = b_dot_n > 0.0 ? b_dot_n * Fb[0] : 0.0;
		}
		return;
	}
	const int iR = P.nc ? P.nc[(size_t)f * NF + i] : i;
	const double* tR = P.traces + (size_t)(2 * f + 1) * NV * NF;
	const double* aR = A.atraces + (size_t)(2 * f + 1) * NV * NF;
#pragma unroll
	for (int k = 0; k < NV; ++k) {
		WL[k] = tL[k * NF + i];
		WR[k] = tR[k * NF + iR];
		// R_L -= E_L^T S F*, R_R += E_R^T S F* (right in its own node order): Fbar = S (E_R xbar_R - E_L xbar_L)
		Fb[k] = sc * (aR[k * NF + iR] - aL[k * NF + i]);
	}
	double* wR = A.wbar + (size_t)(2 * f + 1) * NV * NF;
	if constexpr (PDE == kEuler) {
		double WbL[NV], WbR[NV];
		num_flux_vjp_side<D, NV, FLUX>(WL, WR, n, Fb, 0, WbL);
		num_flux_vjp_side<D, NV, FLUX>(WL, WR, n, Fb, 1, WbR);
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			wL[k * NF + i] = WbL[k];
			wR[k * NF + iR] = WbR[k];
		}
	} else {
		double b_dot_n = 0.0;
#pragma unroll
		for (int k = 0; k < D; ++k)
			b_dot_n += P.b_adv[k] * n[k];
		const bool left = b_dot_n > kEps;   // numerical_flux_advection_T.c:69-72
		wL[i] = left ? b_dot_n * Fb[0] : 0.0;
		wR[iR] = left ? 0.0 : b_dot_n * Fb[0];
	}
}

template <int D, int Q, int NV>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_adj_lift_kernel(const TPOps ops, const TPParams P, const AdjArgs A)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF, E = S::E;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	constexpr int PER_E = 3 * NV * N;
	const int tid = threadIdx.x;
	load_ops(sops, ops);
	const int v0 = blockIdx.x * E;
	const int n_here = min(E, P.n_vol - v0);
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	const int v = v0 + e;
	double* sa = base + e * PER_E;
	double* sb = sa + NV * N;
	double* sc = sb + NV * N;
	__syncthreads();
	if (active) {
		double ub[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			ub[k] = P.vol_gl[((size_t)v * NV + k) * N + node];
#pragma unroll
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int fs = P.vol_face[(size_t)v * 2 * D + lf];
			const int nd = lf >> 1;
			const int a = node_coord<Q>(node, nd);
			int t;
			if (D == 2) {
				t = (nd == 0 ? node_coord<Q>(node, 1) : node_coord<Q>(node, 0));
			} else {
				const int c0 = node_coord<Q>(node, 0), c1 = node_coord<Q>(node, 1), c2 = node_coord<Q>(node, 2);
				t = (nd == 0 ? c1 + Q * c2 : (nd == 1 ? c0 + Q * c2 : c0 + Q * c1));
			}
			const double l = sops->lb[lf & 1][a];
			const double* src = A.wbar + (size_t)fs * NV * NF;   // this side's own node order
#pragma unroll
			for (int k = 0; k < NV; ++k)
				ub[k] += l * src[k * NF + t];
		}
#pragma unroll
		for (int k = 0; k < NV; ++k)
			sa[k * N + node] = ub[k];
	}
	__syncthreads();
	tp_apply<D, Q, NV>(sa, sb, sc, sops->BT, node, active);   // ubar = V^T ubar_g
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			A.ubar[((size_t)v * NV + k) * N + node] = sb[k * N + node];
}

}  // namespace dgpu

namespace dgpu {

// Objective J = sum over the listed faces of the integral of pressure on side 0 (sum_i w_f J_f p(W_L)), and the
// cotangent of side 0's trace, w_f J_f dp/dW, written into wbar (whose other entries the caller zeroes).
template <int D, int NF, int NV>
__global__ void __launch_bounds__(256)
tp_objective_kernel(const TPParams P, const int* __restrict__ faces, int n_obj, double* contrib, double* wbar)
{
	if constexpr (NV != D + 2) {
		return;   // pressure is defined for the Euler equations only (dgpu_set_objective_faces refuses others)
	} else {
	const int gid = blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= n_obj * NF)
		return;
	const int f = faces[gid / NF], i = gid % NF;
	const double* tL = P.traces + (size_t)(2 * f) * NV * NF;
	const double sc = P.fgeo[((size_t)f * (D + 1) + D) * NF + i];
	const double rho = tL[i], E = tL[(D + 1) * NF + i];
	const double rho_inv = 1.0 / rho;
	double V2 = 0.0, u[D];
#pragma unroll
	for (int k = 0; k < D; ++k) {
		u[k] = tL[(1 + k) * NF + i] * rho_inv;
		V2 += u[k] * u[k];
	}
	const double p = kGm1 * (E - 0.5 * rho * V2);
	contrib[gid] = sc * p;
	double* w = wbar + (size_t)(2 * f) * NV * NF;
	w[i] = sc * kGm1 * 0.5 * V2;                       // dp/drho
#pragma unroll
	for (int k = 0; k < D; ++k)
		w[(1 + k) * NF + i] = -sc * kGm1 * u[k];         // dp/dm_k
	w[(D + 1) * NF + i] = sc * kGm1;                   // dp/dE
	}
}

// out = a x + b y + c z (z may be null), elementwise over n doubles.
__global__ void __launch_bounds__(256)
lincomb_kernel(size_t n, double a, const double* x, double b, const double* y, double c, const double* z,
               double* out)
{
	const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	double s = a * x[i] + b * y[i];
	if (z)
		s += c * z[i];
	out[i] = s;
}

}  // namespace dgpu
