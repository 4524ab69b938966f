// Dense-operator residual kernels for the non-tensor-product 3D volumes (TET, WEDGE, PYR) of a batched mesh.
//
// These volumes carry the caller's dense reference operators, as the reference applies its op_std operators with
// one small GEMM per volume (operator_T.c:96-156): s_vc = cv0_vs_vc s (constructor_sol_vc_interp,
// compute_volume_rlhs_T.c:277-285), the contravariant Euler flux at the cubature nodes, rhs = sum_j cv1_j^T
// (w fr_j) (compute_rhs_v_dg_like_T, compute_volume_rlhs_T.c:166-177), face traces cv0_vs_fc s at the face's
// canonical nodes, rhs -= cv0_vs_fc^T (w_f J_f F*) per face (compute_rhs_f_dg_like_T, compute_face_rlhs_T.c:
// 297-310) and M^-1 (scale_rhs_by_m_inv_std, solve_dg.c:265-272). Volumes are affine (constant J), so
// M^-1 = M_ref^-1 / J with M_ref = cv0^T diag(w) cv0 inverted once on the host. A group with a curved volume (J
// varying over the cubature nodes) keeps every volume's own M^-1 instead (dense_minv_kernel).
//
// One CTA handles E volumes of one group; every phase maps one thread to one output row of one volume (all
// variables per thread), reading the operators through the L1 cache (they are shared by every CTA of the group)
// and the volume's state and fluxes from shared memory. The state stays in coefficient space between stages.
#pragma once

#include "dgpu_batched.cuh"

namespace dgpu {

struct DSmem {
	// doubles per element: state (NV n_vs), fluxes (D NV n_vc) and, for a factorised WEDGE, the partial sums of
	// the sum-factorised contractions; the lift keeps its rhs (NV n_vs)
	static __host__ __device__ int vol(int nv, int n_vs, int n_vc) { return nv * n_vs + 3 * nv * n_vc; }
	static __host__ __device__ int prism_tmp(int nv, int n_tvs, int n_tvc, int n_lvs, int n_lvc)
	{
		return nv * (2 * n_lvs * n_tvc + n_lvc * n_tvs);
	}
	static __host__ __device__ int lift(int nv, int n_vs) { return 2 * nv * n_vs + 2; }
};

// Traces of the CTA's volumes (state in shared memory) at each face's canonical nodes.
template <int NV>
__device__ void dtraces(const BParams& P, const DGroup& G, int e0, int n_here, const double* smem, int PER_E)
{
	const int nvs = G.n_vs;
	for (int it = threadIdx.x; it < n_here * G.n_lf * kQMax * kQMax; it += blockDim.x) {
		const int i = it % (kQMax * kQMax), el = it / (kQMax * kQMax), lf = el % G.n_lf, e = el / G.n_lf;
		const long long v = G.elem0 + e0 + e;
		const int4 fd = P.elf[v * kMaxLf + lf];
		const long long fb = P.fbase[fd.x];
		const int nff = (int)(P.fbase[fd.x + 1] - fb);
		if (i >= nff)
			continue;
		const double* op = G.fops + G.fop_off[(lf * G.n_ord + fd.w) * (kQMax + 1) + fd.z] + (long long)i * nvs;
		const double* su = smem + e * PER_E;
		double W[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			W[k] = 0.0;
		for (int m = 0; m < nvs; ++m) {
			const double c = __ldg(op + m);
#pragma unroll
			for (int k = 0; k < NV; ++k)
				W[k] += c * su[k * nvs + m];
		}
		double* dst = P.traces + 2 * NV * fb + (long long)fd.y * NV * nff;
#pragma unroll
		for (int k = 0; k < NV; ++k)
			dst[k * nff + i] = W[k];
	}
}

// Sum-factorised volume term of a WEDGE volume whose operators are Kronecker products of TRI and LINE factors
// (basis index c * n_tvs + t, node index rz * n_tvc + rt): s_vc in two passes (TRI, then LINE), the flux, then
// sum_j cv1_j^T (w fr_j) as LINE then TRI passes for x and y and TRI then LINE for z. Fills sf and vol_gl.
template <int D, int NV, int PDE>
__device__ void dvol_prism_phases(const BParams& P, const DGroup& G, int e0, int n_here, double* smem, int PER_E)
{
	const int nvs = G.n_vs, nvc = G.n_vc, ntv = G.n_tvs, ntc = G.n_tvc, nlv = G.n_lvs, nlc = G.n_lvc;
	const double* __restrict__ T0 = G.tri0;
	const double* __restrict__ T1 = G.tri1;
	const double* __restrict__ L0 = G.line0;
	const double* __restrict__ L1 = G.line1;
	// 1a: v[k][c][rt] = sum_t T0[rt][t] s[k][c][t]
	for (int it = threadIdx.x; it < n_here * NV * nlv * ntc; it += blockDim.x) {
		const int e = it / (NV * nlv * ntc), rem = it % (NV * nlv * ntc);
		const int k = rem / (nlv * ntc), c = (rem / ntc) % nlv, rt = rem % ntc;
		const double* su = smem + e * PER_E + k * nvs + c * ntv;
		const double* row = T0 + (long long)rt * ntv;
		double acc = 0.0;
		for (int t = 0; t < ntv; ++t)
			acc += __ldg(row + t) * su[t];
		smem[e * PER_E + NV * nvs + 3 * NV * nvc + rem] = acc;
	}
	__syncthreads();
	// 1b: W[k] at (rz, rt) = sum_c L0[rz][c] v[k][c][rt]; the flux there
	for (int it = threadIdx.x; it < n_here * nvc; it += blockDim.x) {
		const int e = it / nvc, r = it % nvc, rz = r / ntc, rt = r % ntc;
		const double* v = smem + e * PER_E + NV * nvs + 3 * NV * nvc;
		double* sf = smem + e * PER_E + NV * nvs;
		double W[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			double acc = 0.0;
			for (int c = 0; c < nlv; ++c)
				acc += __ldg(L0 + rz * nlv + c) * v[(k * nlv + c) * ntc + rt];
			W[k] = acc;
		}
		double g[D * D];
		const double* gm = P.gmet + G.gmet_off + (long long)(e0 + e) * D * D * nvc;
#pragma unroll
		for (int cc = 0; cc < D * D; ++cc)
			g[cc] = gm[cc * nvc + r];
		if constexpr (PDE == kEuler) {
			double fr[D][D + 2];
			euler_flux_ref<D>(W, g, fr);
#pragma unroll
			for (int j = 0; j < D; ++j)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					sf[(j * NV + k) * nvc + r] = fr[j][k];
		} else {
#pragma unroll
			for (int j = 0; j < D; ++j) {
				double gb = 0.0;
#pragma unroll
				for (int i = 0; i < D; ++i)
					gb += g[j * D + i] * P.b_adv[i];
				sf[j * nvc + r] = gb * W[0];
			}
		}
	}
	__syncthreads();
	// 2a: gx, gy[k][c][rt] = sum_rz L0[rz][c] f_x,y[k][rz][rt];  h[k][rz][t] = sum_rt T0[rt][t] f_z[k][rz][rt]
	const int gsz = NV * nlv * ntc;
	for (int it = threadIdx.x; it < n_here * gsz; it += blockDim.x) {
		const int e = it / gsz, rem = it % gsz;
		const int k = rem / (nlv * ntc), c = (rem / ntc) % nlv, rt = rem % ntc;
		const double* sf = smem + e * PER_E + NV * nvs;
		double* tmp = smem + e * PER_E + NV * nvs + 3 * NV * nvc;
		double ax = 0.0, ay = 0.0;
		for (int rz = 0; rz < nlc; ++rz) {
			const double l = __ldg(L0 + rz * nlv + c);
			ax += l * sf[(0 * NV + k) * nvc + rz * ntc + rt];
			ay += l * sf[(1 * NV + k) * nvc + rz * ntc + rt];
		}
		tmp[rem] = ax;
		tmp[gsz + rem] = ay;
	}
	const int hsz = NV * nlc * ntv;
	for (int it = threadIdx.x; it < n_here * hsz; it += blockDim.x) {
		const int e = it / hsz, rem = it % hsz;
		const int k = rem / (nlc * ntv), rz = (rem / ntv) % nlc, t = rem % ntv;
		const double* fz = smem + e * PER_E + NV * nvs + (2 * NV + k) * nvc + rz * ntc;
		double* h = smem + e * PER_E + NV * nvs + 3 * NV * nvc + 2 * gsz;
		double acc = 0.0;
		for (int rt = 0; rt < ntc; ++rt)
			acc += __ldg(T0 + (long long)rt * ntv + t) * fz[rt];
		h[rem] = acc;
	}
	__syncthreads();
	// 2b: vol[k][c][t] = sum_rt (T1x[rt][t] gx[k][c][rt] + T1y[rt][t] gy[k][c][rt]) + sum_rz L1[rz][c] h[k][rz][t]
	for (int it = threadIdx.x; it < n_here * NV * nvs; it += blockDim.x) {
		const int e = it / (NV * nvs), rem = it % (NV * nvs), k = rem / nvs, c = (rem % nvs) / ntv, t = rem % ntv;
		const double* tmp = smem + e * PER_E + NV * nvs + 3 * NV * nvc;
		const double* gx = tmp + (k * nlv + c) * ntc;
		const double* gy = gx + gsz;
		const double* h = tmp + 2 * gsz + k * nlc * ntv + t;
		double acc = 0.0;
		for (int rt = 0; rt < ntc; ++rt)
			acc += __ldg(T1 + (long long)rt * ntv + t) * gx[rt] + __ldg(T1 + (long long)(ntc + rt) * ntv + t) * gy[rt];
		for (int rz = 0; rz < nlc; ++rz)
			acc += __ldg(L1 + rz * nlv + c) * h[rz * ntv];
		P.vol_gl[G.state_off + (long long)(e0 + e) * NV * nvs + rem] = acc;
	}
}

// ---------------------------------------------------------------------------------------------------------------
// Volume term (coefficient space) + face traces at the canonical face nodes
// ---------------------------------------------------------------------------------------------------------------
template <int D, int NV, int PDE>
__device__ void dvol_body(const BParams& P, const DGroup& G, int e0, int E, const double* __restrict__ u,
                          double* smem)
{
	const int nvs = G.n_vs, nvc = G.n_vc;
	const int PER_E = G.vol_per_e;
	const int n_here = min(E, G.n_vol - e0);
	const double* ublk = u + G.state_off + (long long)e0 * NV * nvs;
	for (int i = threadIdx.x; i < n_here * NV * nvs; i += blockDim.x) {
		const int e = i / (NV * nvs), r = i % (NV * nvs);
		smem[e * PER_E + r] = ublk[i];
	}
	__syncthreads();
	if (G.prism) {
		dvol_prism_phases<D, NV, PDE>(P, G, e0, n_here, smem, PER_E);
		dtraces<NV>(P, G, e0, n_here, smem, PER_E);
		__syncthreads();   // shared memory is reused by the next tile
		return;
	}
	const double* __restrict__ cv0 = G.cv0;
	// phase 1: state at the cubature nodes, contravariant flux, w-weighted (w is folded into the metrics)
	for (int it = threadIdx.x; it < n_here * nvc; it += blockDim.x) {
		const int e = it / nvc, r = it % nvc;
		const double* su = smem + e * PER_E;
		double* sf = smem + e * PER_E + NV * nvs;   // [j][k][r]
		double W[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			W[k] = 0.0;
		const double* row = cv0 + (long long)r * nvs;
		for (int m = 0; m < nvs; ++m) {
			const double c = __ldg(row + m);
#pragma unroll
			for (int k = 0; k < NV; ++k)
				W[k] += c * su[k * nvs + m];
		}
		double g[D * D];
		const double* gm = P.gmet + G.gmet_off + (long long)(e0 + e) * D * D * nvc;
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			g[c] = gm[c * nvc + r];
		if constexpr (PDE == kEuler) {
			double fr[D][D + 2];
			euler_flux_ref<D>(W, g, fr);
#pragma unroll
			for (int j = 0; j < D; ++j)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					sf[(j * NV + k) * nvc + r] = fr[j][k];
		} else {
#pragma unroll
			for (int j = 0; j < D; ++j) {
				double gb = 0.0;
#pragma unroll
				for (int i = 0; i < D; ++i)
					gb += g[j * D + i] * P.b_adv[i];
				sf[j * nvc + r] = gb * W[0];
			}
		}
	}
	__syncthreads();
	// phase 2: rhs_vol[k][m] = sum_j sum_r cv1_j[r][m] sf[j][k][r]
	const double* __restrict__ cv1 = G.cv1;
	for (int it = threadIdx.x; it < n_here * NV * nvs; it += blockDim.x) {
		const int e = it / (NV * nvs), rem = it % (NV * nvs), k = rem / nvs, m = rem % nvs;
		const double* sf = smem + e * PER_E + NV * nvs;
		double acc = 0.0;
#pragma unroll
		for (int j = 0; j < D; ++j) {
			const double* col = cv1 + (long long)j * nvc * nvs + m;
			const double* f = sf + (j * NV + k) * nvc;
			for (int r = 0; r < nvc; ++r)
				acc += __ldg(col + (long long)r * nvs) * f[r];
		}
		P.vol_gl[G.state_off + (long long)(e0 + e) * NV * nvs + k * nvs + m] = acc;
	}
	dtraces<NV>(P, G, e0, n_here, smem, PER_E);
	__syncthreads();   // shared memory is reused by the next tile
}

// ---------------------------------------------------------------------------------------------------------------
// Lift of the face fluxes, M^-1, then the residual or the RK stage (coefficient space)
// ---------------------------------------------------------------------------------------------------------------
// enforce_positivity_highorder (solve.c:187-233) on the new states of the CTA's elements (kept at NV n_vs of
// each element's block): Bezier coefficients b = ccSB0 s per variable; one thread per element converts them to
// primitive variables, checks the average (error flag below EPS_PHYS) and minimum of the density, then of the
// pressure, and when a minimum is below EPS_PHYS blends every variable toward its average (correct_coef,
// :356-374) before the pressure check; corrected elements get s = ccBS0 b back in conserved variables. Elements
// that need no correction keep s (the reference's round trip is the identity up to rounding).
template <int NV>
__device__ void dense_positivity(const BParams& P, const DGroup& G, int e0, int n_here, const RkArgs& rk,
                                 double* smem, int PER_E)
{
	constexpr double kEpsPhys = 1e-13;   // definitions_tol.h EPS_PHYS
	constexpr int D = NV - 2;
	const int nvs = G.n_vs;
	__syncthreads();
	// FP32 pre-filter: per element the scales S_k = max |s_k| (into the free rhs half), then every Bezier node's
	// density and pressure lower bounds from FP32 coefficients and their rounding bound pos_err S_k; an element
	// whose bounds all clear the thresholds (which lie far above EPS_PHYS) needs no correction and is skipped
	// the state in FP32 once (after the NV scales in the free rhs half), so the n_vs^2 products run on FP32 only
	for (int it = threadIdx.x; it < n_here * NV * nvs; it += blockDim.x) {
		const int e = it / (NV * nvs), rem = it % (NV * nvs);
		reinterpret_cast<float*>(smem + e * PER_E + NV)[rem] = (float)smem[e * PER_E + NV * nvs + rem];
	}
	for (int it = threadIdx.x; it < n_here * NV; it += blockDim.x) {   // one thread per (volume, variable)
		const int e = it / NV, k = it % NV;
		const double* sv = smem + e * PER_E + NV * nvs + k * nvs;
		double mx = 0.0;
		for (int a = 0; a < nvs; ++a)
			mx = fmax(mx, fabs(sv[a]));
		smem[e * PER_E + k] = mx;
		if (k == 0)
			smem[e * PER_E + 2 * NV * nvs + 1] = 0.0;   // unsafe flag
	}
	__syncthreads();
	for (int it = threadIdx.x; it < n_here * nvs; it += blockDim.x) {
		const int e = it / nvs, m = it % nvs;
		const float* sf = reinterpret_cast<const float*>(smem + e * PER_E + NV);
		const float* row = G.ccSB0f + (long long)m * nvs;
		float bk[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			float acc = 0.f;
			for (int a = 0; a < nvs; ++a)
				acc += __ldg(row + a) * sf[k * nvs + a];
			bk[k] = acc;
		}
		const float err = G.pos_err;
		const float s_rho = (float)smem[e * PER_E];
		const float rho_lo = bk[0] - err * s_rho;
		bool safe = rho_lo > 1e-6f * s_rho + 1e-12f;
		if (safe) {
			float m2 = 0.f;
#pragma unroll
			for (int d = 0; d < D; ++d) {
				const float mk = fabsf(bk[1 + d]) + err * (float)smem[e * PER_E + 1 + d];
				m2 += mk * mk;
			}
			const float E_lo = bk[D + 1] - err * (float)smem[e * PER_E + D + 1];
			const float ke = 0.5f * m2 / rho_lo;
			const float p_lo = 0.4f * (E_lo - ke);
			safe = p_lo > 1e-5f * (fabsf(E_lo) + ke) + 1e-12f;   // NaN/Inf fail this test and go to the exact path
		}
		if (!safe)
			smem[e * PER_E + 2 * NV * nvs + 1] = 1.0;
	}
	__syncthreads();
	for (int it = threadIdx.x; it < n_here * NV * nvs; it += blockDim.x) {
		const int e = it / (NV * nvs), rem = it % (NV * nvs), k = rem / nvs, m = rem % nvs;
		if (smem[e * PER_E + 2 * NV * nvs + 1] == 0.0)
			continue;
		const double* sv = smem + e * PER_E + NV * nvs + k * nvs;
		const double* row = G.ccSB0 + (long long)m * nvs;
		double b = 0.0;
		for (int a = 0; a < nvs; ++a)
			b += __ldg(row + a) * sv[a];
		smem[e * PER_E + rem] = b;
	}
	__syncthreads();
	// conserved -> primitive (rho, u, p) at every Bezier node (convert_variables 'c' -> 'p'), node-parallel
	for (int it = threadIdx.x; it < n_here * nvs; it += blockDim.x) {
		const int e = it / nvs, m = it % nvs;
		if (smem[e * PER_E + 2 * NV * nvs + 1] == 0.0)
			continue;
		double* b = smem + e * PER_E;
		const double rho = b[m];
		double V2 = 0.0;
#pragma unroll
		for (int d = 0; d < D; ++d) {
			const double u = b[(1 + d) * nvs + m] / rho;
			b[(1 + d) * nvs + m] = u;
			V2 += u * u;
		}
		b[(D + 1) * nvs + m] = kGm1 * (b[(D + 1) * nvs + m] - 0.5 * rho * V2);
	}
	__syncthreads();
	// per element: the rhs half of its block now holds b, the other half s; the flag takes a spare scalar slot
	for (int e = threadIdx.x; e < n_here; e += blockDim.x) {
		double* b = smem + e * PER_E;
		bool corrected = false;
		if (smem[e * PER_E + 2 * NV * nvs + 1] == 0.0) {   // cleared by the pre-filter
			smem[e * PER_E + 2 * NV * nvs] = 0.0;
			continue;
		}
		for (int vr = 0; vr < NV; vr += NV - 1) {
			double avg = 0.0, mn = b[vr * nvs];
			for (int m = 0; m < nvs; ++m) {
				avg += b[vr * nvs + m];
				mn = fmin(mn, b[vr * nvs + m]);
			}
			avg /= nvs;
			if (!(avg >= kEpsPhys)) {
				atomicExch(P.err_flag, 1);
				break;
			}
			if (mn < kEpsPhys) {
				const double th = fmax(0.0, fmin(1.0, (avg - kEpsPhys) / (avg - mn)));
				for (int k = 0; k < NV; ++k) {
					double a = 0.0;
					for (int m = 0; m < nvs; ++m)
						a += b[k * nvs + m];
					a /= nvs;
					if ((k == 0 || k == NV - 1) && a < kEpsPhys)
						a = kEpsPhys;
					for (int m = 0; m < nvs; ++m)
						b[k * nvs + m] = th * b[k * nvs + m] + (1.0 - th) * a;
				}
				corrected = true;
			}
		}
		if (corrected)
			atomicAdd(P.n_corr, 1ull);
		smem[e * PER_E + 2 * NV * nvs] = corrected ? 1.0 : 0.0;
	}
	__syncthreads();
	// primitive -> conserved on the corrected elements, node-parallel
	for (int it = threadIdx.x; it < n_here * nvs; it += blockDim.x) {
		const int e = it / nvs, m = it % nvs;
		if (smem[e * PER_E + 2 * NV * nvs] == 0.0)
			continue;
		double* b = smem + e * PER_E;
		const double rho = b[m];
		double V2 = 0.0;
#pragma unroll
		for (int d = 0; d < D; ++d) {
			const double u = b[(1 + d) * nvs + m];
			V2 += u * u;
			b[(1 + d) * nvs + m] = rho * u;
		}
		b[(D + 1) * nvs + m] = b[(D + 1) * nvs + m] / kGm1 + 0.5 * rho * V2;
	}
	__syncthreads();
	for (int it = threadIdx.x; it < n_here * NV * nvs; it += blockDim.x) {
		const int e = it / (NV * nvs), rem = it % (NV * nvs), k = rem / nvs, m = rem % nvs;
		if (smem[e * PER_E + 2 * NV * nvs] == 0.0)
			continue;
		const double* bv = smem + e * PER_E + k * nvs;
		const double* row = G.ccBS0 + (long long)m * nvs;
		double s = 0.0;
		for (int a = 0; a < nvs; ++a)
			s += __ldg(row + a) * bv[a];
		rk.u[G.state_off + (long long)(e0 + e) * NV * nvs + rem] = s;
	}
}

template <int NV, int MODE>
__device__ void dlift_body(const BParams& P, const DGroup& G, int e0, int E, const RkArgs& rk, double* smem)
{
	const int nvs = G.n_vs;
	const int PER_E = G.lift_per_e;
	const int n_here = min(E, G.n_vol - e0);
	// phase 1: rhs = vol - sum_lf sgn cv0_fc^T nnf
	for (int it = threadIdx.x; it < n_here * NV * nvs; it += blockDim.x) {
		const int e = it / (NV * nvs), rem = it % (NV * nvs), k = rem / nvs, m = rem % nvs;
		const long long v = G.elem0 + e0 + e;
		double acc = P.vol_gl[G.state_off + (long long)(e0 + e) * NV * nvs + rem];
		if (P.source)   // cv0^T diag(w J) s
			acc += P.source[G.state_off + (long long)(e0 + e) * NV * nvs + rem];
		for (int lf = 0; lf < G.n_lf; ++lf) {
			const int4 fd = P.elf[v * kMaxLf + lf];
			const long long fb = P.fbase[fd.x];
			const int nff = (int)(P.fbase[fd.x + 1] - fb);
			const double* op = G.fops + G.fop_off[(lf * G.n_ord + fd.w) * (kQMax + 1) + fd.z] + m;
			const double* src = P.nnf + NV * fb + (long long)k * nff;
			// side 1 reads the face flux (side 0's node order) at its own nodes through the inverse permutation
			const int* ci = (fd.y == 1 && P.nc_inv) ? P.nc_inv + fb : nullptr;
			double s = 0.0;
			for (int i = 0; i < nff; ++i)
				s += __ldg(op + (long long)i * nvs) * src[ci ? ci[i] : i];
			acc += (fd.y == 0 ? -s : s);   // side 0: rhs -= ; side 1: rhs -= (-nnf)
		}
		smem[e * PER_E + rem] = acc;
	}
	__syncthreads();
	// phase 2: R = M_ref^-1 rhs / J, then the stage
	const double* __restrict__ minv = G.minv;
	unsigned long long mx = 0ull;
	for (int it = threadIdx.x; it < n_here * NV * nvs; it += blockDim.x) {
		const int e = it / (NV * nvs), rem = it % (NV * nvs), k = rem / nvs, m = rem % nvs;
		const double* sr = smem + e * PER_E + k * nvs;
		double R;
		if (G.minv_vol) {   // curved volumes: the volume's own M^-1
			const double* row = G.minv_vol + ((long long)(e0 + e) * nvs + m) * nvs;
			R = 0.0;
			for (int a = 0; a < nvs; ++a)
				R += __ldg(row + a) * sr[a];
		} else {
			if (G.minv_identity) {
				R = sr[m];
			} else {
				const double* row = minv + (long long)m * nvs;
				R = 0.0;
				for (int a = 0; a < nvs; ++a)
					R += __ldg(row + a) * sr[a];
			}
			R *= G.inv_J[e0 + e];
		}
		const long long o = G.state_off + (long long)(e0 + e) * NV * nvs + rem;
		if (MODE == kModeRhs || rk.want_max) {
			const unsigned long long bits = abs_bits(R);
			mx = bits > mx ? bits : mx;
		}
		if constexpr (MODE == kModeRhs) {
			rk.rhs[o] = R;
		} else {
			const double s = rk.u[o];
			double sn;
			if (rk.stage == 0) {
				rk.u0[o] = s;
				sn = s + rk.dt * R;
			} else if (rk.stage == 1) {
				sn = (1.0 / 4.0) * (3.0 * rk.u0[o] + s + rk.dt * R);
			} else {
				sn = (1.0 / 3.0) * (rk.u0[o] + 2.0 * s + 2.0 * rk.dt * R);
			}
			rk.u[o] = sn;
			smem[e * PER_E + NV * nvs + rem] = sn;   // kept for the positivity check
		}
	}
	if constexpr (MODE != kModeRhs) {
		if (rk.positivity && G.ccSB0)
			dense_positivity<NV>(P, G, e0, n_here, rk, smem, PER_E);
	}
	if (MODE == kModeRhs || rk.want_max) {
#pragma unroll
		for (int off = 16; off > 0; off >>= 1) {
			const unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, off);
			mx = o > mx ? o : mx;
		}
		if ((threadIdx.x & 31) == 0 && mx && P.max_bits)
			atomicMax(P.max_bits, mx);
	}
	__syncthreads();   // shared memory is reused by the next tile
}

// ---------------------------------------------------------------------------------------------------------------
// Kernels: one launch per dense group, and the bodies the fused kernels dispatch to
// ---------------------------------------------------------------------------------------------------------------

// Shared memory of dense_minv_kernel: the augmented matrix [M | I] (n_vs x 2 n_vs) and one column.
__host__ __device__ inline size_t dense_minv_smem(int nvs) { return (size_t)(2 * nvs * nvs + nvs) * sizeof(double); }

// M^-1 of one curved volume per CTA (set-up, once per context): M = cv0^T diag(w J) cv0 (constructor_mass_T,
// volume_solver_T.c:115-145) formed in shared memory, then inverted by Gauss-Jordan elimination. M is symmetric
// positive definite, so the pivots (Schur complements) are positive and no row exchange is needed.
// cv0: n_vc x n_vs; wJ: per volume n_vc values w_n J_n; minv: per volume n_vs x n_vs row-major.
__global__ void __launch_bounds__(128) dense_minv_kernel(const double* __restrict__ cv0,
                                                         const double* __restrict__ wJ, int nvs, int nvc,
                                                         int n_vol, double* __restrict__ minv)
{
	extern __shared__ double sm[];
	const int v = blockIdx.x;
	if (v >= n_vol)
		return;
	const int w2 = 2 * nvs;
	double* A = sm;                // [M | I]
	double* col = sm + nvs * w2;   // column k before elimination step k
	const double* wj = wJ + (long long)v * nvc;
	for (int it = threadIdx.x; it < nvs * nvs; it += blockDim.x) {
		const int a = it / nvs, b = it % nvs;
		double s = 0.0;
		for (int r = 0; r < nvc; ++r)
			s += cv0[(long long)r * nvs + a] * wj[r] * cv0[(long long)r * nvs + b];
		A[a * w2 + b] = s;
		A[a * w2 + nvs + b] = (a == b) ? 1.0 : 0.0;
	}
	__syncthreads();
	for (int k = 0; k < nvs; ++k) {
		for (int i = threadIdx.x; i < nvs; i += blockDim.x)
			col[i] = A[i * w2 + k];
		__syncthreads();
		const double inv_p = 1.0 / col[k];
		for (int j = threadIdx.x; j < w2; j += blockDim.x)
			A[k * w2 + j] *= inv_p;
		__syncthreads();
		for (int it = threadIdx.x; it < nvs * w2; it += blockDim.x) {
			const int i = it / w2, j = it - i * w2;
			if (i != k)
				A[i * w2 + j] -= col[i] * A[k * w2 + j];
		}
		__syncthreads();
	}
	for (int it = threadIdx.x; it < nvs * nvs; it += blockDim.x) {
		const int a = it / nvs, b = it % nvs;
		minv[((long long)v * nvs + a) * nvs + b] = A[a * w2 + nvs + b];
	}
}

template <int D, int NV, int PDE>
__global__ void __launch_bounds__(256) dvol_group_kernel(const BParams P, int g, const double* __restrict__ u)
{
	extern __shared__ double smem[];
	const DGroup G = P.dgroups[g];
	if (blockIdx.x == 0 && threadIdx.x == 0 && P.max_bits && G.elem0 == 0)
		*P.max_bits = 0ull;
	dvol_body<D, NV, PDE>(P, G, blockIdx.x * G.E, G.E, u, smem);
}

template <int NV, int MODE>
__global__ void __launch_bounds__(256) dlift_group_kernel(const BParams P, int g, const RkArgs rk)
{
	extern __shared__ double smem[];
	const DGroup G = P.dgroups[g];
	dlift_body<NV, MODE>(P, G, blockIdx.x * G.E, G.E, rk, smem);
}

// Fused persistent kernels: a CTA walks the tile list (grid-stride) and dispatches on the tile's group: a TP
// group's order (its operator set is reloaded into shared memory when the group changes) or a dense group.
// Each (group kind, q) body is called as a separate function (not inlined): the kernel then needs the registers
// of its largest body, not those of all bodies inlined into one switch.
template <int D, int Q, int NV, int PDE, bool GLL_IN>
__device__ __noinline__ void bvol_tile(const BParams& P, const BatchOps* sops, const BGroup& G, int e0, int E,
                                       const double* __restrict__ u, double* base)
{
	bvol_body<D, Q, NV, PDE, GLL_IN>(P, sops, G, e0, E, u, base);
}

template <int D, int NV, int PDE>
__device__ __noinline__ void dvol_tile(const BParams& P, const DGroup& G, int e0, int E, const double* __restrict__ u,
                                       double* base)
{
	dvol_body<D, NV, PDE>(P, G, e0, E, u, base);
}

template <int D, int Q, int NV, int MODE>
__device__ __noinline__ void blift_tile(const BParams& P, const BatchOps* sops, const BGroup& G, int e0, int E,
                                        const RkArgs& rk, double* base)
{
	blift_body<D, Q, NV, MODE>(P, sops, G, e0, E, rk, base);
}

template <int NV, int MODE>
__device__ __noinline__ void dlift_tile(const BParams& P, const DGroup& G, int e0, int E, const RkArgs& rk,
                                        double* base)
{
	dlift_body<NV, MODE>(P, G, e0, E, rk, base);
}

template <int D, int NV, int PDE, bool GLL_IN>
__global__ void __launch_bounds__(256) bvol_fused_kernel(const BParams P, const BTile* tiles, int n_tiles,
                                                           const double* __restrict__ u)
{
	extern __shared__ double smem[];
	BatchOps* sops = reinterpret_cast<BatchOps*>(smem);
	double* base = smem + sizeof(BatchOps) / 8;
	if (blockIdx.x == 0 && threadIdx.x == 0 && P.max_bits)
		*P.max_bits = 0ull;
	int cur = -1;
	for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
		const BTile tl = tiles[t];
		if (tl.group >= P.n_groups) {
			const DGroup G = P.dgroups[tl.group - P.n_groups];
			dvol_tile<D, NV, PDE>(P, G, tl.e0, G.E_fused, u, base);
			continue;
		}
		if (tl.group != cur) {
			__syncthreads();
			load_batch_ops(sops, &P.ops[tl.group]);
			cur = tl.group;
			__syncthreads();
		}
		const BGroup G = P.groups[tl.group];
		const int E = (int)(blockDim.x / (D == 2 ? G.q * G.q : G.q * G.q * G.q));
		switch (G.q) {
		case 2: bvol_tile<D, 2, NV, PDE, GLL_IN>(P, sops, G, tl.e0, E, u, base); break;
		case 3: bvol_tile<D, 3, NV, PDE, GLL_IN>(P, sops, G, tl.e0, E, u, base); break;
		case 4: bvol_tile<D, 4, NV, PDE, GLL_IN>(P, sops, G, tl.e0, E, u, base); break;
		default: bvol_tile<D, 5, NV, PDE, GLL_IN>(P, sops, G, tl.e0, E, u, base); break;
		}
	}
}

// The RK stages that reduce no max |rhs| run the TP tiles without that path (as the per-group form does), capped at
// 4 CTAs per SM; the dense tiles take the want_max flag at run time.
template <int D, int NV, int MODE>
__global__ void __launch_bounds__(256, BLiftOccupancy<MODE>::value) blift_fused_kernel(const BParams P,
                                                                                     const BTile* tiles, int n_tiles,
                                                                                     const RkArgs rk)
{
	constexpr int DMODE = (MODE == kModeRkGlNoMax) ? kModeRkGl : MODE;
	extern __shared__ double smem[];
	BatchOps* sops = reinterpret_cast<BatchOps*>(smem);
	double* base = smem + sizeof(BatchOps) / 8;
	int cur = -1;
	for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
		const BTile tl = tiles[t];
		if (tl.group >= P.n_groups) {
			const DGroup G = P.dgroups[tl.group - P.n_groups];
			dlift_tile<NV, DMODE>(P, G, tl.e0, G.E_fused, rk, base);
			continue;
		}
		if (tl.group != cur) {
			__syncthreads();
			load_batch_ops(sops, &P.ops[tl.group]);
			cur = tl.group;
			__syncthreads();
		}
		const BGroup G = P.groups[tl.group];
		const int E = (int)(blockDim.x / (D == 2 ? G.q * G.q : G.q * G.q * G.q));
		switch (G.q) {
		case 2: blift_tile<D, 2, NV, MODE>(P, sops, G, tl.e0, E, rk, base); break;
		case 3: blift_tile<D, 3, NV, MODE>(P, sops, G, tl.e0, E, rk, base); break;
		case 4: blift_tile<D, 4, NV, MODE>(P, sops, G, tl.e0, E, rk, base); break;
		default: blift_tile<D, 5, NV, MODE>(P, sops, G, tl.e0, E, rk, base); break;
		}
	}
}

// ---------------------------------------------------------------------------------------------------------------
// Form 3: a whole stage in one cooperative persistent launch (volume tiles | face nodes | lift tiles)
// ---------------------------------------------------------------------------------------------------------------
// Barrier between the phases over every CTA of the grid. The launch is cooperative, so all CTAs are resident at
// once and the barrier completes; each wait is still bounded (limit_ns of the global timer, 2 s by default): a CTA
// that gives up sets *err = kErrBarrier and returns false, and the kernel then ends. bar[0] counts the arrivals of
// the current barrier and bar[1] its generation; the host zeroes both before each launch.
constexpr int kErrBarrier = 2;
constexpr unsigned long long kBarrierLimitNs = 2000000000ull;

__device__ __forceinline__ unsigned long long global_ns()
{
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* err, unsigned long long limit_ns)
{
	__shared__ int ok;
	__syncthreads();   // the CTA's writes of this phase are issued
	if (threadIdx.x == 0) {
		ok = 1;
		volatile unsigned* gen = bar + 1;
		const unsigned g = *gen;   // cannot advance before this CTA arrives
		__threadfence();           // this CTA's writes are visible before its arrival
		if (atomicAdd(bar, 1u) == gridDim.x - 1) {
			atomicExch(bar, 0u);
			__threadfence();
			atomicAdd(bar + 1, 1u);
		} else {
			const unsigned long long t0 = global_ns();
			while (*gen == g) {
				if (global_ns() - t0 > limit_ns) {
					atomicExch(err, kErrBarrier);
					ok = 0;
					break;
				}
				__nanosleep(64);
			}
		}
		__threadfence();
	}
	__syncthreads();
	return ok != 0;
}

// The three phases of the fused form in one kernel: the volume tiles, every face node of the q_f-sorted list, the
// lift tiles; grid barriers in between. One occupancy serves all three phases: the shared memory of the largest
// tile (the q = 2 volume tile in 3D, 82 KB) already limits it to 2 CTAs per SM, so registers are capped there too
// (a 64-register cap would only add spills).
template <int D, int NV, int PDE, int FLUX, int MODE, bool GLL_IN>
__global__ void __launch_bounds__(256, 2)
bstage_kernel(const BParams P, const BTile* __restrict__ tiles, int n_tiles, const double* __restrict__ u,
              const int* __restrict__ node_face, long long n_nodes, const RkArgs rk, unsigned* bar,
              unsigned long long limit_ns)
{
	constexpr int DMODE = (MODE == kModeRkGlNoMax) ? kModeRkGl : MODE;
	extern __shared__ double smem[];
	BatchOps* sops = reinterpret_cast<BatchOps*>(smem);
	double* base = smem + sizeof(BatchOps) / 8;
	if (blockIdx.x == 0 && threadIdx.x == 0 && P.max_bits)
		*P.max_bits = 0ull;
	int cur = -1;
	for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
		const BTile tl = tiles[t];
		if (tl.group >= P.n_groups) {
			const DGroup G = P.dgroups[tl.group - P.n_groups];
			dvol_tile<D, NV, PDE>(P, G, tl.e0, G.E_fused, u, base);
			continue;
		}
		if (tl.group != cur) {
			__syncthreads();
			load_batch_ops(sops, &P.ops[tl.group]);
			cur = tl.group;
			__syncthreads();
		}
		const BGroup G = P.groups[tl.group];
		const int E = (int)(blockDim.x / (D == 2 ? G.q * G.q : G.q * G.q * G.q));
		switch (G.q) {
		case 2: bvol_tile<D, 2, NV, PDE, GLL_IN>(P, sops, G, tl.e0, E, u, base); break;
		case 3: bvol_tile<D, 3, NV, PDE, GLL_IN>(P, sops, G, tl.e0, E, u, base); break;
		case 4: bvol_tile<D, 4, NV, PDE, GLL_IN>(P, sops, G, tl.e0, E, u, base); break;
		default: bvol_tile<D, 5, NV, PDE, GLL_IN>(P, sops, G, tl.e0, E, u, base); break;
		}
	}
	if (!grid_barrier(bar, P.err_flag, limit_ns))
		return;
	for (long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x; gid < n_nodes;
	     gid += (long long)gridDim.x * blockDim.x) {
		const int f = node_face[gid];
		const long long fb = P.fbase[f];
		bface_node_rt<D, NV, PDE, FLUX>(P, f, (int)(gid - fb), (int)(P.fbase[f + 1] - fb));
	}
	if (!grid_barrier(bar, P.err_flag, limit_ns))
		return;
	for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
		const BTile tl = tiles[t];
		if (tl.group >= P.n_groups) {
			const DGroup G = P.dgroups[tl.group - P.n_groups];
			dlift_tile<NV, DMODE>(P, G, tl.e0, G.E_fused, rk, base);
			continue;
		}
		if (tl.group != cur) {
			__syncthreads();
			load_batch_ops(sops, &P.ops[tl.group]);
			cur = tl.group;
			__syncthreads();
		}
		const BGroup G = P.groups[tl.group];
		const int E = (int)(blockDim.x / (D == 2 ? G.q * G.q : G.q * G.q * G.q));
		switch (G.q) {
		case 2: blift_tile<D, 2, NV, MODE>(P, sops, G, tl.e0, E, rk, base); break;
		case 3: blift_tile<D, 3, NV, MODE>(P, sops, G, tl.e0, E, rk, base); break;
		case 4: blift_tile<D, 4, NV, MODE>(P, sops, G, tl.e0, E, rk, base); break;
		default: blift_tile<D, 5, NV, MODE>(P, sops, G, tl.e0, E, rk, base); break;
		}
	}
}

// Face numerical flux at every node of the faces in [node_lo, node_hi) of the q_f-sorted face node list.
template <int D, int NV, int PDE, int FLUX>
__global__ void __launch_bounds__(256) bface_nodes_kernel(const BParams P, const int* __restrict__ node_face,
                                                           long long node_lo, long long node_hi)
{
	for (long long gid = node_lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; gid < node_hi;
	     gid += (long long)gridDim.x * blockDim.x) {
		const int f = node_face[gid];
		const long long fb = P.fbase[f];
		bface_node_rt<D, NV, PDE, FLUX>(P, f, (int)(gid - fb), (int)(P.fbase[f + 1] - fb));
	}
}

}  // namespace dgpu
