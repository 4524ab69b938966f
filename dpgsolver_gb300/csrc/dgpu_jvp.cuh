// Forward-mode linearisation of the residual: R(u) and the directional derivative (dR/du) du in one pass.
//
// The reference linearises its residual by complex step (compute_lhs_cmplx_step_dg,
// src/testing/support/simulation/solvers/dg/test_support_solve_dg.c:83-110): every flux routine is instantiated for
// double complex and the imaginary part of R(u + i h du) / h is the product. Here the flux routines are
// instantiated for the dual number Dual<1> (value, derivative), which gives the same product without the step h.
// Everything between the fluxes is linear (V, Dgl^T, the traces, the lift, diag(1/(wJ)), V^-1), so the tangent
// rides through those as a second set of buffers: the volume and face kernels below write the primal quantities to
// the primal parameter set P and the tangent ones to Pd, and the ordinary lift kernel in residual mode, run once on
// P and once on Pd, finishes R and (dR/du) du.
#pragma once

#include "dgpu_tp.cuh"

namespace dgpu {

// Volume term on GLL coefficients u (primal) and du (tangent): both through V, the flux as Dual<1>, the
// contraction and the traces of each. Per element: 2 x (su, st, sf) in shared memory.
template <int D, int Q, int NV, int PDE>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_jvp_volume_kernel(const TPOps ops, const TPParams P, const TPParams Pd, const double* __restrict__ u,
                     const double* __restrict__ du)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF, E = S::E;
	constexpr int VOL = TPSmem<D, Q, NV>::VOL;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	load_ops(sops, ops);
	const int tid = threadIdx.x;
	const int v0 = blockIdx.x * E;
	const int n_here = min(E, P.n_vol - v0);
	for (int i = tid; i < n_here * NV * N; i += blockDim.x) {
		const int e = i / (NV * N), r = i % (NV * N);
		base[(2 * e) * VOL + r] = u[(size_t)v0 * NV * N + i];
		base[(2 * e + 1) * VOL + r] = du[(size_t)v0 * NV * N + i];
	}
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* su = base + (2 * e) * VOL;
	double* st = su + NV * N;
	double* sf = st + NV * N;
	double* dsu = base + (2 * e + 1) * VOL;
	double* dst = dsu + NV * N;
	double* dsf = dst + NV * N;
	// ug = V u and dug = V du (su and dsu receive the GL values)
	tp_apply<D, Q, NV>(su, st, sf, sops->B, node, active);
	tp_apply<D, Q, NV>(dsu, dst, dsf, sops->B, node, active);
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			su[k * N + node] = st[k * N + node];
			dsu[k * N + node] = dst[k * N + node];
		}
	__syncthreads();
	const int v = v0 + e;
	if (active) {
		double g[D * D];
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			g[c] = P.gmet[((size_t)v * D * D + c) * N + node];
		if constexpr (PDE == kEuler) {
			Dual<1> W[NV];
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				W[k].v = su[k * N + node];
				W[k].d[0] = dsu[k * N + node];
			}
			Dual<1> fr[D][D + 2];
			euler_flux_ref<D, Dual<1>>(W, g, fr);
#pragma unroll
			for (int j = 0; j < D; ++j)
#pragma unroll
				for (int k = 0; k < NV; ++k) {
					sf[(j * NV + k) * N + node] = fr[j][k].v;
					dsf[(j * NV + k) * N + node] = fr[j][k].d[0];
				}
		} else {
#pragma unroll
			for (int j = 0; j < D; ++j) {
				double gb = 0.0;
#pragma unroll
				for (int i = 0; i < D; ++i)
					gb += g[j * D + i] * P.b_adv[i];
				sf[j * N + node] = gb * su[node];
				dsf[j * N + node] = gb * dsu[node];
			}
		}
	}
	__syncthreads();
	if (!active)
		return;
	// contraction sum_j Dgl_j^T (w fr_j) of the flux and of its derivative
	double acc[NV], dacc[NV];
#pragma unroll
	for (int k = 0; k < NV; ++k)
		acc[k] = dacc[k] = 0.0;
#pragma unroll
	for (int j = 0; j < D; ++j) {
		const int stride = (j == 0 ? 1 : (j == 1 ? Q : Q * Q));
		const int a = node_coord<Q>(node, j);
		const int b0 = node - a * stride;
#pragma unroll
		for (int m = 0; m < Q; ++m) {
			const double w = sops->Dgl[m][a];
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				acc[k] += w * sf[(j * NV + k) * N + b0 + m * stride];
				dacc[k] += w * dsf[(j * NV + k) * N + b0 + m * stride];
			}
		}
	}
#pragma unroll
	for (int k = 0; k < NV; ++k) {
		P.vol_gl[((size_t)v * NV + k) * N + node] = acc[k];
		Pd.vol_gl[((size_t)v * NV + k) * N + node] = dacc[k];
	}
	// traces of both on the 2D local faces
	for (int it = node; it < 2 * D * NF; it += N) {
		const int lf = it / NF, t = it % NF;
		const int nd = lf >> 1, side = lf & 1;
		const int t0 = (D == 2 ? t : t % Q), t1 = (D == 2 ? 0 : t / Q);
		int stride_n, base_n;
		if (D == 2) {
			stride_n = (nd == 0 ? 1 : Q);
			base_n = (nd == 0 ? t0 * Q : t0);
		} else {
			stride_n = (nd == 0 ? 1 : (nd == 1 ? Q : Q * Q));
			base_n = (nd == 0 ? t0 * Q + t1 * Q * Q : (nd == 1 ? t0 + t1 * Q * Q : t0 + t1 * Q));
		}
		const int fs = P.vol_face[(size_t)v * 2 * D + lf];
		double* dst_p = P.traces + (size_t)fs * NV * NF;
		double* dst_d = Pd.traces + (size_t)fs * NV * NF;
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			double s = 0.0, ds = 0.0;
#pragma unroll
			for (int m = 0; m < Q; ++m) {
				const double l = sops->lb[side][m];
				s += l * su[k * N + base_n + m * stride_n];
				ds += l * dsu[k * N + base_n + m * stride_n];
			}
			dst_p[k * NF + t] = s;
			dst_d[k * NF + t] = ds;
		}
	}
}

// Numerical flux at every face node of the primal traces (P) and its derivative along the tangent traces (Pd).
template <int D, int Q, int NV, int PDE, int FLUX>
__global__ void __launch_bounds__(256) tp_jvp_face_kernel(const TPParams P, const TPParams Pd)
{
	using S = TPShape<D, Q>;
	constexpr int NF = S::NF;
	const int gid = blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= P.n_face * NF)
		return;
	const int f = gid / NF, i = gid % NF;
	const int b = P.bnd ? P.bnd[f] : -1;
	const int iR = P.nc ? P.nc[(size_t)f * NF + i] : i;
	const size_t oL = (size_t)(2 * f) * NV * NF, oR = (size_t)(2 * f + 1) * NV * NF;
	double n[D];
	const double* fg = P.fgeo + (size_t)f * (D + 1) * NF;
#pragma unroll
	for (int k = 0; k < D; ++k)
		n[k] = fg[k * NF + i];
	const double sc = fg[D * NF + i];
	double* out = P.nnf + (size_t)f * NV * NF;
	double* dout = Pd.nnf + (size_t)f * NV * NF;
	if constexpr (PDE == kEuler) {
		Dual<1> WL[NV], WR[NV], nF[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			WL[k].v = P.traces[oL + k * NF + i];
			WL[k].d[0] = Pd.traces[oL + k * NF + i];
		}
		if (b < 0) {
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				WR[k].v = P.traces[oR + k * NF + iR];
				WR[k].d[0] = Pd.traces[oR + k * NF + iR];
			}
		} else {
			boundary_value<D, NV, PDE, Dual<1>>(P, b, i, NF, WL, n, WR);
		}
		if constexpr (FLUX == kRoePike)
			num_flux_roe_pike<D, Dual<1>>(WL, WR, n, nF);
		else
			num_flux_lax_friedrichs<D, Dual<1>>(WL, WR, n, nF);
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			out[k * NF + i] = nF[k].v * sc;
			dout[k * NF + i] = nF[k].d[0] * sc;
		}
	} else {
		// upwind: linear in the traces, the branch set by b.n alone; the boundary value is the interior trace
		// (derivative: its tangent) or the fixed exterior state (derivative 0)
		double uR = 0.0, duR = 0.0;
		if (b < 0) {
			uR = P.traces[oR + iR];
			duR = Pd.traces[oR + iR];
		} else {
			Dual<1> uL, r;
			uL.v = P.traces[oL + i];
			uL.d[0] = Pd.traces[oL + i];
			boundary_value<D, NV, PDE, Dual<1>>(P, b, i, NF, &uL, n, &r);
			uR = r.v;
			duR = r.d[0];
		}
		out[i] = num_flux_upwind<D>(P.traces[oL + i], uR, n, P.b_adv) * sc;
		dout[i] = num_flux_upwind<D>(Pd.traces[oL + i], duR, n, P.b_adv) * sc;
	}
}

}  // namespace dgpu
