// Tensor-product (QUAD/HEX) explicit DG residual kernels for sm_103a, FP64.
//
// Formulation. The reference applies dense per-element operators (operator_T.c:96-156 -> cblas_dgemm):
//   R = M^-1 [ sum_d tw1_vt_vc[d] fr_d - sum_faces tw0_vt_fc nnf ],   M = V^T diag(w J) V,
// with V = cv0_vs_vc. On TP elements with GLL solution nodes and (p+1)-point GL cubature V = B (x) B (x) B is
// square and invertible (B = 1D GLL->GL interpolation), cv1_vs_vc[d] = Dgl_d V (GL collocation derivative,
// exact for degree p), and cv0_vs_fc[lf] = E_lf V (E_lf = GL Lagrange values at the face). Hence
//   R = V^-1 R_gl,   R_gl = diag(1/(w J)) [ sum_d Dgl_d^T (w fr_d) - sum_lf E_lf^T (w_f J_f F*) ],
// the same operator in exact arithmetic with the V^-T V^T pair cancelled: every contraction is a 1D
// sum-factorised pass of q FMAs per node, and the dense per-element M^-1 is never formed.
//
// Because the SSP-RK3 stage update is linear, V u_new = a V u0 + b (V u + dt R) = a ug0 + b (ug + dt R_gl): the
// time stepper keeps the state as GL nodal values ug = V u and never applies V or V^-1 inside a step; the
// reference's GLL coefficients are recovered (V^-1) only when the caller reads the state.
//
// Kernels:
//   tp_volume_kernel   [V u ->] ug; Euler/advection flux and metric contraction; sum_j Dgl_j^T; face traces.
//   tp_face_kernel     per face node: numerical flux of the two traces, scaled by w_f J_f.
//   tp_lift_kernel     lift of the face fluxes and diag(1/(wJ)); then either V^-1 + residual + max|rhs| (the
//                      reference's compute_rhs_dg), or the RK stage update in GL space + positivity check.
//   tp_convert_kernel  u <-> ug.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dgpu_physics.cuh"

namespace dgpu {

constexpr int kQMax = 5;  // p <= 4

// 1D operators of one (element type, p), derived on the host from the caller's ops_tp factors.
struct TPOps {
	double B[kQMax][kQMax];     // GLL -> GL interpolation  B[m][a]
	double Binv[kQMax][kQMax];  // GL -> GLL                 Binv[a][m]
	double Dgl[kQMax][kQMax];   // GL collocation derivative Dgl[m][k] = l_k'(x_m)
	double lb[2][kQMax];        // GL Lagrange basis at r = -1 / +1
	double SB[kQMax][kQMax];    // ccSB0 1D (Lagrange -> Bezier)
	double BS[kQMax][kQMax];    // ccBS0 1D (Bezier -> Lagrange)
	double SBg[kQMax][kQMax];   // ccSB0 B^-1: GL nodal values -> Bezier coefficients
	double BSg[kQMax][kQMax];   // B ccBS0:   Bezier coefficients -> GL nodal values
	double BT[kQMax][kQMax];    // B^T    (adjoint: V^T)
	double BinvT[kQMax][kQMax]; // Binv^T (adjoint: V^-T)
	float SBf[kQMax][kQMax];    // SBg rounded to FP32 (positivity pre-filter)
	float pos_err;              // |FP32 Bezier coefficient - exact| <= pos_err * max_i |x_i| (per variable)
};
static_assert(sizeof(TPOps) % 8 == 0, "TPOps is copied to shared memory as doubles");

struct TPParams {
	int n_vol;
	int n_face;
	double b_adv[3];
	const int* vol_face;       // [v][2D]: face * 2 + side
	const double* gmet;        // [v][D*D][N]: w_vc * metrics, component j*D+i = w J dr_j/dx_i
	const double* inv_wJ;      // [v][N]: 1 / (w_vc J_vc)
	const double* fgeo;        // [f][D+1][NF]: unit normal (D) and w_fc J_f
	const int* nc;             // [f][NF] right-trace gather permutation, or nullptr (identity)
	const int* nc_inv;         // [f][NF] its inverse, or nullptr
	double* traces;            // [f][2][NV][NF]
	double* nnf;               // [f][NV][NF]
	double* vol_gl;            // [v][NV][N]
	unsigned long long* max_bits;  // max |rhs| as the bit pattern of a non-negative double
	int* err_flag;             // positivity failure flag
	unsigned long long* n_corr;    // positivity corrections applied
	// Boundary faces (no side-1 volume), or all three nullptr on a mesh without any:
	const int* bnd;            // [f] index b of the face in the boundary list, -1 for an interior face
	const int* bc_code;        // [b] BC code modulo BC_STEP_SC
	const double* bc_ext;      // [b][NV][NF] exterior (test case) conserved state at the face nodes
	BcData bc_data;            // back pressure / total temperature and pressure data
	// Navier-Stokes (BR2 second-order terms), all nullptr otherwise:
	double* ns_gtr;            // [face side][D][NV][NF] traces of the volume gradient
	const double* ns_lam;      // [face side][NF] diagonal of the face's own lifting at its nodes
	double* ns_X;              // [f][D][NV][NF] w_f J_f n (s_R - s_L) / 2, side-0 node order
	double* ns_gv;             // [v][D][NV][N] volume gradient (physical, at the GL nodes)
	NsPhys ns;                 // viscosity model and constants
	double ns_eta;             // BR2 scaling of a face's own lifting in its face gradient
	// Volume kernel on GLL coefficients only (may be null): also keep the coefficients it read and the GL values it
	// formed, so that one pass over a caller's host buffer both uploads the state and starts the RK step.
	double* keep_coef = nullptr;   // [v][NV][N]
	double* keep_gl = nullptr;     // [v][NV][N]
	// The test case's source term at the volume cubature nodes, or null (compute_source_rhs_dg_like,
	// src/simulation/solvers/compute_rlhs.c:47-57). M^-1 tw0_vt_vc (J s) = V^-1 s on the GL nodes, so it adds to the
	// GL nodal residual after the 1/(w J) scaling.
	const double* source = nullptr;   // [v][NV][N]
};

// Right-hand state of face node i of boundary face b: the boundary value of its BC from the interior trace WL.
template <int D, int NV, int PDE, typename T>
__device__ __forceinline__ void boundary_value(const TPParams& P, int b, int i, int NF, const T* WL, const double* n,
                                               T* WR)
{
	const double* ext = P.bc_ext + (size_t)b * NV * NF;
	if constexpr (PDE == kEuler) {
		double e[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			e[k] = ext[k * NF + i];
		euler_boundary_state<D, T>(P.bc_code[b], WL, e, n, WR, P.bc_data);
	} else {
		WR[0] = advection_boundary_value<D, T>(WL[0], ext[i], n, P.b_adv);
	}
}

template <int D, int Q>
struct TPShape {
	static constexpr int N = (D == 2 ? Q * Q : Q * Q * Q);
	static constexpr int NF = (D == 2 ? Q : Q * Q);
	static constexpr int E = (N >= 256 ? 1 : 256 / N);   // elements per CTA
	static constexpr int THREADS = ((E * N + 31) / 32) * 32;  // whole warps; surplus threads idle
};

// Index of the node along direction `dir`.
template <int Q>
__device__ __forceinline__ int node_coord(int node, int dir)
{
	return dir == 0 ? node % Q : (dir == 1 ? (node / Q) % Q : node / (Q * Q));
}

// One sum-factorised pass along `dir`: out[var][node] = sum_m M[a(node)][m] in[var][node with a -> m].
template <int D, int Q, int NV, typename T, typename TM>
__device__ __forceinline__ void tp_pass(const T* __restrict__ in, T* __restrict__ out, const TM (*M)[kQMax],
                                        int dir, int node)
{
	constexpr int N = TPShape<D, Q>::N;
	const int stride = (dir == 0 ? 1 : (dir == 1 ? Q : Q * Q));
	const int a = node_coord<Q>(node, dir);
	const int base = node - a * stride;
	T w[Q];
#pragma unroll
	for (int m = 0; m < Q; ++m)
		w[m] = (T)M[a][m];
#pragma unroll
	for (int v = 0; v < NV; ++v) {
		T s = 0;
#pragma unroll
		for (int m = 0; m < Q; ++m)
			s += w[m] * in[v * N + base + m * stride];
		out[v * N + node] = s;
	}
}

// The D passes of M (x) M (x) M over one element block: in -> out, `tmp` as scratch (in, out, tmp distinct).
// Every thread of the CTA must call it (it synchronises); `active` selects the threads that compute.
template <int D, int Q, int NV, typename T, typename TM>
__device__ __forceinline__ void tp_apply(const T* in, T* out, T* tmp, const TM (*M)[kQMax], int node, bool active)
{
	if (D == 2) {
		if (active) tp_pass<D, Q, NV>(in, tmp, M, 0, node);
		__syncthreads();
		if (active) tp_pass<D, Q, NV>(tmp, out, M, 1, node);
	} else {
		if (active) tp_pass<D, Q, NV>(in, out, M, 0, node);
		__syncthreads();
		if (active) tp_pass<D, Q, NV>(out, tmp, M, 1, node);
		__syncthreads();
		if (active) tp_pass<D, Q, NV>(tmp, out, M, 2, node);
	}
	__syncthreads();
}

__device__ __forceinline__ unsigned long long abs_bits(double x)
{
	return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

// Copies the operator set into shared memory; the caller synchronises before use.
__device__ __forceinline__ void load_ops(TPOps* sops, const TPOps& ops)
{
	for (int i = threadIdx.x; i < (int)(sizeof(TPOps) / 8); i += blockDim.x)
		reinterpret_cast<double*>(sops)[i] = reinterpret_cast<const double*>(&ops)[i];
}

// ---------------------------------------------------------------------------------------------------------------
// Volume term + traces
// ---------------------------------------------------------------------------------------------------------------
// Shared memory per element of the bodies below (doubles).
template <int D, int Q, int NV>
struct TPSmem {
	static constexpr int N = TPShape<D, Q>::N;
	static constexpr int VOL = NV * N * 2 + D * NV * N;   // su, st, sf
	static constexpr int LIFT = 3 * NV * N + 8;           // sa, sb, sc, per-element scalars
};

// Volume term of the CTA's E elements; per element PER_E doubles at base (su, st, sf at the start).
template <int D, int Q, int NV, int PDE, bool GLL_IN, int PER_E>
__device__ __forceinline__ void tp_volume_body(const TPOps* sops, const TPParams& P, const double* __restrict__ u,
                                               int v0, int n_here, double* base)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF;
	const int tid = threadIdx.x;
	for (int i = tid; i < n_here * NV * N; i += blockDim.x) {   // coalesced: contiguous element blocks
		const int e = i / (NV * N), r = i % (NV * N);
		const double x = u[(size_t)v0 * NV * N + i];
		base[e * PER_E + r] = x;
		if (GLL_IN && P.keep_coef)
			P.keep_coef[(size_t)v0 * NV * N + i] = x;
	}
	__syncthreads();

	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* su = base + e * PER_E;
	double* st = su + NV * N;
	double* sf = st + NV * N;

	if (GLL_IN) {
		// ug = V u: passes su -> st (-> sf) -> ... ; copy into su so the traces and flux read one buffer
		tp_apply<D, Q, NV>(su, st, sf, sops->B, node, active);
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				su[k * N + node] = st[k * N + node];
				if (P.keep_gl)
					P.keep_gl[((size_t)(v0 + e) * NV + k) * N + node] = st[k * N + node];
			}
		__syncthreads();
	}

	const int v = v0 + e;
	if (active) {
		double W[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			W[k] = su[k * N + node];
		double g[D * D];
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			g[c] = P.gmet[((size_t)v * D * D + c) * N + node];
		if constexpr (PDE == kEuler) {
			double fr[D][D + 2];
			euler_flux_ref<D>(W, g, fr);
#pragma unroll
			for (int j = 0; j < D; ++j)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					sf[(j * NV + k) * N + node] = fr[j][k];
		} else {
			// advection: f_i = b_i u ; fr_j = sum_i g[j][i] b_i u
#pragma unroll
			for (int j = 0; j < D; ++j) {
				double gb = 0.0;
#pragma unroll
				for (int i = 0; i < D; ++i)
					gb += g[j * D + i] * P.b_adv[i];
				sf[j * N + node] = gb * W[0];
			}
		}
	}
	__syncthreads();

	if (active) {
		// volume term in GL space: sum_j Dgl_j^T (w fr_j)
		double acc[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			acc[k] = 0.0;
#pragma unroll
		for (int j = 0; j < D; ++j) {
			const int stride = (j == 0 ? 1 : (j == 1 ? Q : Q * Q));
			const int a = node_coord<Q>(node, j);
			const int b0 = node - a * stride;
			double w[Q];
#pragma unroll
			for (int m = 0; m < Q; ++m)
				w[m] = sops->Dgl[m][a];
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				const double* f = sf + (j * NV + k) * N + b0;
#pragma unroll
				for (int m = 0; m < Q; ++m)
					acc[k] += w[m] * f[m * stride];
			}
		}
#pragma unroll
		for (int k = 0; k < NV; ++k)
			P.vol_gl[((size_t)v * NV + k) * N + node] = acc[k];

		// traces of ug on the 2D local faces
		for (int it = node; it < 2 * D * NF; it += N) {
			const int lf = it / NF, t = it % NF;
			const int nd = lf >> 1, side = lf & 1;
			int t0, t1;
			if (D == 2) {
				t0 = t; t1 = 0;
			} else {
				t0 = t % Q; t1 = t / Q;
			}
			// node index with coordinate m along nd and tangential (t0, t1) in ascending direction order
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
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				double s = 0.0;
#pragma unroll
				for (int m = 0; m < Q; ++m)
					s += sops->lb[side][m] * su[k * N + base_n + m * stride_n];
				dst[k * NF + t] = s;
			}
		}
	}
}

template <int D, int Q, int NV, int PDE, bool GLL_IN>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_volume_kernel(const TPOps ops, const TPParams P, const double* __restrict__ u)
{
	using S = TPShape<D, Q>;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	load_ops(sops, ops);
	const int v0 = blockIdx.x * S::E;
	if (blockIdx.x == 0 && threadIdx.x == 0 && P.max_bits)
		*P.max_bits = 0ull;
	tp_volume_body<D, Q, NV, PDE, GLL_IN, TPSmem<D, Q, NV>::VOL>(sops, P, u, v0, min(S::E, P.n_vol - v0),
	                                                                   smem + sizeof(TPOps) / 8);
}

// ---------------------------------------------------------------------------------------------------------------
// Face numerical flux
// ---------------------------------------------------------------------------------------------------------------
template <int D, int Q, int NV, int PDE, int FLUX>
__global__ void __launch_bounds__(256)
tp_face_kernel(const TPParams P)
{
	using S = TPShape<D, Q>;
	constexpr int NF = S::NF;
	const int gid = blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= P.n_face * NF)
		return;
	const int f = gid / NF, i = gid % NF;
	const int b = P.bnd ? P.bnd[f] : -1;
	const double* tL = P.traces + (size_t)(2 * f) * NV * NF;
	double WL[NV], WR[NV], n[D];
#pragma unroll
	for (int k = 0; k < NV; ++k)
		WL[k] = tL[k * NF + i];
	const double* fg = P.fgeo + (size_t)f * (D + 1) * NF;
#pragma unroll
	for (int k = 0; k < D; ++k)
		n[k] = fg[k * NF + i];
	if (b < 0) {
		const int iR = P.nc ? P.nc[(size_t)f * NF + i] : i;
		const double* tR = P.traces + (size_t)(2 * f + 1) * NV * NF;
#pragma unroll
		for (int k = 0; k < NV; ++k)
			WR[k] = tR[k * NF + iR];
	} else {
		boundary_value<D, NV, PDE, double>(P, b, i, NF, WL, n, WR);
	}
	const double sc = fg[D * NF + i];
	double* out = P.nnf + (size_t)f * NV * NF;
	if constexpr (PDE == kEuler) {
		double nF[NV];
		if constexpr (FLUX == kRoePike) {
			num_flux_roe_pike<D>(WL, WR, n, nF);
#pragma unroll
			for (int k = 0; k < NV; ++k)
				nF[k] *= sc;
		} else {
			num_flux_lax_friedrichs<D>(WL, WR, n, nF, sc);
		}
#pragma unroll
		for (int k = 0; k < NV; ++k)
			out[k * NF + i] = nF[k];
	} else {
		out[i] = num_flux_upwind<D>(WL[0], WR[0], n, P.b_adv) * sc;
	}
}

// ---------------------------------------------------------------------------------------------------------------
// Lift + M^-1 + (residual | RK stage + positivity)
// ---------------------------------------------------------------------------------------------------------------
// kModeRkGl reads rk.want_max at run time; kModeRkGlNoMax is the RK stage compiled without the max |rhs| path
// (fewer registers for the common graph-replayed stage).
// kModeRkGlOut is kModeRkGl that also writes the new state's GLL coefficients (the last stage of a step whose result
// goes back to the caller).
enum LiftMode { kModeRhs = 0, kModeRkGl = 1, kModeRkGlNoMax = 2, kModeRkGlOut = 3 };

struct RkArgs {
	double* u;         // kModeRkGl: state as GL nodal values (ug), updated in place
	double* u0;        // kModeRkGl: stage-0 copy (ug of sol_coef_p)
	double* rhs;       // kModeRhs: residual output (GLL coefficients)
	double dt;
	int stage;         // 0, 1, 2
	int positivity;
	int want_max;      // kModeRkGl: also reduce max |rhs| (needs V^-1 of the GL residual)
	double* out_coef = nullptr;   // kModeRkGlOut: V^-1 of the new state (GLL coefficients)
	double* out_host = nullptr;   // kModeRkGlOut: the same into a caller's pinned host buffer, or null
};

// enforce_positivity_highorder (solve.c:187-233) on one element held in shared memory.
// `c` holds the element's conserved state [NV][N] in the basis that `toB` maps to Bezier coefficients (`fromB`
// maps back); `b` and `tmp` are scratch [NV][N]. Returns true when this element was corrected (c then holds the
// corrected state). The reference's serial averages and minima run on one thread per element; the Bezier
// transforms are sum-factorised passes by the element's threads. All threads of the CTA must call it.
template <int D, int Q, int NV>
__device__ __noinline__ bool tp_positivity_exact(const double (*toB)[kQMax], const double (*fromB)[kQMax], double* c, double* b,
                                    double* tmp, int node, bool active, int* flag_out)
{
	constexpr int N = TPShape<D, Q>::N;
	tp_apply<D, Q, NV>(c, b, tmp, toB, node, active);
	// convert_variables c -> p per coefficient (solution_euler_T.c:173-194)
	if (active) {
		const double rho = b[node];
		const double rho_inv = 1.0 / rho;
		double rho2V2 = 0.0;
#pragma unroll
		for (int k = 0; k < D; ++k) {
			const double m = b[(1 + k) * N + node];
			rho2V2 += m * m;
			b[(1 + k) * N + node] = m * rho_inv;
		}
		b[(D + 1) * N + node] = kGm1 * (b[(D + 1) * N + node] - 0.5 * rho2V2 * rho_inv);
	}
	__syncthreads();
	int corrected = 0;
	if (active && node == 0) {
		for (int vr = 0; vr < NV; vr += NV - 1) {
			const double* vd = b + vr * N;
			double s = 0.0, mn = vd[0];
			for (int i = 0; i < N; ++i) {
				s += vd[i];
				if (vd[i] < mn)
					mn = vd[i];
			}
			const double avg = s / N;
			if (avg < kEpsPhys) {
				*flag_out = 1;
				break;
			}
			if (mn < kEpsPhys) {
				double p_ho = (avg - kEpsPhys) / (avg - mn);
				p_ho = fmax(0.0, fmin(1.0, p_ho));
				// correct_coef (solve.c:356-374)
				for (int w = 0; w < NV; ++w) {
					double* data = b + w * N;
					double aw = 0.0;
					for (int i = 0; i < N; ++i)
						aw += data[i];
					aw /= N;
					if ((w == 0 || w == NV - 1) && aw < kEpsPhys)
						aw = kEpsPhys;
					for (int i = 0; i < N; ++i)
						data[i] = p_ho * data[i] + (1 - p_ho) * aw;
				}
				corrected = 1;
			}
		}
		tmp[0] = corrected;  // broadcast through shared memory (tmp is free here)
	}
	__syncthreads();
	corrected = active ? (int)tmp[0] : 0;
	__syncthreads();
	const int any = __syncthreads_or(corrected);
	if (!any)
		return false;
	if (corrected) {
		// convert p -> c per coefficient, then back to the state's basis
		const double rho = b[node];
		double V2 = 0.0;
#pragma unroll
		for (int k = 0; k < D; ++k) {
			const double uu = b[(1 + k) * N + node];
			V2 += uu * uu;
			b[(1 + k) * N + node] = rho * uu;
		}
		b[(D + 1) * N + node] = b[(D + 1) * N + node] / kGm1 + 0.5 * rho * V2;
	}
	__syncthreads();
	tp_apply<D, Q, NV>(b, c, tmp, fromB, node, corrected != 0);
	return corrected != 0;
}

// Positivity in the RK epilogue. The exact check is the reference's FP64 computation above. It is preceded by
// an FP32 pre-filter that proves, for most elements, that the exact check cannot trigger: every FP32 Bezier
// coefficient carries an absolute error of at most pos_err * max_i |x_i| of its variable (a forward bound for D
// passes of q-term FMA dot products with FP32-rounded inputs and coefficients, computed on the host with a factor
// 2 margin); density and pressure are bounded below from those intervals, with a further relative margin of
// 1e-5 on the pressure bound for its own FP32 arithmetic. Only CTAs holding an element that fails the filter run
// the exact check, so the decisions are those of the exact FP64 check.

// Lift, 1/(wJ), then the residual (V^-1, max|rhs|) or the RK stage + positivity, for the CTA's E elements; per
// element PER_E doubles at base.
template <int D, int Q, int NV, int MODE, int PER_E>
__device__ __forceinline__ void tp_lift_body(const TPOps* sops, const TPParams& P, const RkArgs& rk, int v0,
                                             int n_here, double* base)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF;
	const int tid = threadIdx.x;
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	const int v = v0 + e;
	double* sa = base + e * PER_E;
	double* sb = sa + NV * N;
	double* sc = sb + NV * N;
	int* sscale = reinterpret_cast<int*>(sc + NV * N);   // NV ints (FP32 scales) + spare
	if (active && node < 8)
		reinterpret_cast<double*>(sscale)[node] = 0.0;
	__syncthreads();  // the lift below reads sops->lb written by other warps

	double Rg[NV];  // GL-space residual R_gl of this node
	if (active) {
#pragma unroll
		for (int k = 0; k < NV; ++k)
			Rg[k] = P.vol_gl[((size_t)v * NV + k) * N + node];
#pragma unroll
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int fs = P.vol_face[(size_t)v * 2 * D + lf];
			const int f = fs >> 1, s = fs & 1;
			const int nd = lf >> 1;
			const int a = node_coord<Q>(node, nd);
			int t;
			if (D == 2) {
				t = (nd == 0 ? node_coord<Q>(node, 1) : node_coord<Q>(node, 0));
			} else {
				const int c0 = node_coord<Q>(node, 0), c1 = node_coord<Q>(node, 1), c2 = node_coord<Q>(node, 2);
				t = (nd == 0 ? c1 + Q * c2 : (nd == 1 ? c0 + Q * c2 : c0 + Q * c1));
			}
			const int idx = (s == 1 && P.nc_inv) ? P.nc_inv[(size_t)f * NF + t] : t;
			// side 0: rhs -= E^T nnf ; side 1: rhs -= E^T (-nnf)   (compute_face_rlhs_T.c:297-310)
			const double l = (s == 0 ? -1.0 : 1.0) * sops->lb[lf & 1][a];
			const double* src = P.nnf + (size_t)f * NV * NF;
#pragma unroll
			for (int k = 0; k < NV; ++k)
				Rg[k] += l * src[k * NF + idx];
		}
		const double iw = P.inv_wJ[(size_t)v * N + node];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			Rg[k] *= iw;
		if (P.source)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				Rg[k] += P.source[((size_t)v * NV + k) * N + node];
	}

	const bool need_coef = (MODE == kModeRhs) || ((MODE == kModeRkGl || MODE == kModeRkGlOut) && rk.want_max);
	unsigned long long mx = 0ull;
	double R[NV];
	if (MODE != kModeRkGlNoMax && need_coef) {
		// R = V^-1 R_gl (GLL coefficients): D passes of Binv
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				sa[k * N + node] = Rg[k];
		__syncthreads();
		tp_apply<D, Q, NV>(sa, sb, sc, sops->Binv, node, active);
		if (active) {
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				R[k] = sb[k * N + node];
				const unsigned long long bits = abs_bits(R[k]);
				mx = bits > mx ? bits : mx;
			}
		}
		// max |rhs| (compute_max_rhs_dg_like): integer max over the bit patterns of |R|
#pragma unroll
		for (int off = 16; off > 0; off >>= 1) {
			const unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, off);
			mx = o > mx ? o : mx;
		}
		if ((tid & 31) == 0 && mx && P.max_bits)
			atomicMax(P.max_bits, mx);
		__syncthreads();   // sa/sb/sc are reused below
	}

	if constexpr (MODE == kModeRhs) {
		if (active) {
#pragma unroll
			for (int k = 0; k < NV; ++k)
				rk.rhs[((size_t)v * NV + k) * N + node] = R[k];
		}
		return;
	} else {
		// SSP-RK3 stage update in GL space (solve_explicit.c:277-295; linear, so V commutes with it)
		double snew[NV];
		if (active) {
			const size_t o = (size_t)v * NV * N + node;
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				const double s = rk.u[o + (size_t)k * N];
				if (rk.stage == 0) {
					rk.u0[o + (size_t)k * N] = s;
					snew[k] = s + rk.dt * Rg[k];
				} else if (rk.stage == 1) {
					const double sp = rk.u0[o + (size_t)k * N];
					snew[k] = (1.0 / 4.0) * (3.0 * sp + s + rk.dt * Rg[k]);
				} else {
					const double sp = rk.u0[o + (size_t)k * N];
					snew[k] = (1.0 / 3.0) * (sp + 2.0 * s + 2.0 * rk.dt * Rg[k]);
				}
			}
		}
		if (rk.positivity) {
			if (active)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					sb[k * N + node] = snew[k];
			__syncthreads();
			// FP32 pre-filter (sa as float [NV][N] x2, sscale per element)
			float* xf = reinterpret_cast<float*>(sa);
			float* tf = xf + NV * N;
			float* tmpf = reinterpret_cast<float*>(sc);
			if (active) {
#pragma unroll
				for (int k = 0; k < NV; ++k) {
					const float x = (float)snew[k];
					xf[k * N + node] = x;
					atomicMax(&sscale[k], __float_as_int(fabsf(x)));
				}
			}
			__syncthreads();
			tp_apply<D, Q, NV>(xf, tf, tmpf, sops->SBf, node, active);
			bool safe = true;
			if (active) {
				const float err = sops->pos_err;
				const float rho = tf[node];
				const float erho = err * __int_as_float(sscale[0]);
				const float rho_lo = rho - erho;
				safe = rho_lo > 1e-6f * __int_as_float(sscale[0]) + 1e-12f;
				if (safe) {
					float m2 = 0.f;
#pragma unroll
					for (int k = 0; k < D; ++k) {
						const float mk = fabsf(tf[(1 + k) * N + node]) + err * __int_as_float(sscale[1 + k]);
						m2 += mk * mk;
					}
					const float E_lo = tf[(D + 1) * N + node] - err * __int_as_float(sscale[D + 1]);
					const float ke = 0.5f * m2 / rho_lo;
					const float p_lo = 0.4f * (E_lo - ke);
					const float mag = fabsf(E_lo) + ke;
					safe = p_lo > 1e-5f * mag + 1e-12f;   // NaN/Inf fail this test and go to the exact path
				}
			}
			const int unsafe = __syncthreads_or(active && !safe);
			if (unsafe) {
				int flag = 0;
				const bool corr =
					tp_positivity_exact<D, Q, NV>(sops->SBg, sops->BSg, sb, sc, sa, node, active, &flag);
				if (flag)
					atomicExch(P.err_flag, 1);
				if (corr) {
					if (node == 0)
						atomicAdd(P.n_corr, 1ull);
#pragma unroll
					for (int k = 0; k < NV; ++k)
						snew[k] = sb[k * N + node];
				}
			}
		}
		if (active) {
			const size_t o = (size_t)v * NV * N + node;
#pragma unroll
			for (int k = 0; k < NV; ++k)
				rk.u[o + (size_t)k * N] = snew[k];
		}
		if constexpr (MODE == kModeRkGlOut) {
			// the new state's GLL coefficients: V^-1 of the GL values (D passes of Binv)
			__syncthreads();   // sa/sb/sc are free again
			if (active)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					sa[k * N + node] = snew[k];
			__syncthreads();
			tp_apply<D, Q, NV>(sa, sb, sc, sops->Binv, node, active);
			if (active)
#pragma unroll
				for (int k = 0; k < NV; ++k) {
					const size_t o = ((size_t)v * NV + k) * N + node;
					rk.out_coef[o] = sb[k * N + node];
					if (rk.out_host)
						rk.out_host[o] = sb[k * N + node];
				}
		}
	}
}

// Minimum CTAs per SM of the lift kernel (caps its registers): 3 for the plain RK stage, 2 otherwise.
template <int MODE>
struct LiftOccupancy { static constexpr int value = (MODE == kModeRkGlNoMax) ? 4 : 2; };   // Out: as RkGl

template <int D, int Q, int NV, int MODE>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS, LiftOccupancy<MODE>::value)
tp_lift_kernel(const TPOps ops, const TPParams P, const RkArgs rk)
{
	using S = TPShape<D, Q>;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	load_ops(sops, ops);
	const int v0 = blockIdx.x * S::E;
	tp_lift_body<D, Q, NV, MODE, TPSmem<D, Q, NV>::LIFT>(sops, P, rk, v0, min(S::E, P.n_vol - v0),
	                                                            smem + sizeof(TPOps) / 8);
}

// ---------------------------------------------------------------------------------------------------------------
// u (GLL coefficients) <-> ug (GL nodal values)
// ---------------------------------------------------------------------------------------------------------------
// in_copy / out_copy (either may be null): also write the input / the result there, so that one pass both moves a
// state between a caller's pinned host buffer and the device and changes its basis.
template <int D, int Q, int NV, bool TO_GL>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_convert_kernel(const TPOps ops, int n_vol, const double* __restrict__ in, double* __restrict__ out,
                  double* __restrict__ in_copy, double* __restrict__ out_copy)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, E = S::E;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	constexpr int PER_E = 3 * NV * N;
	const int tid = threadIdx.x;
	load_ops(sops, ops);
	const int v0 = blockIdx.x * E;
	const int n_here = min(E, n_vol - v0);
	for (int i = tid; i < n_here * NV * N; i += blockDim.x) {
		const int e = i / (NV * N), r = i % (NV * N);
		const double x = in[(size_t)v0 * NV * N + i];
		base[e * PER_E + r] = x;
		if (in_copy)
			in_copy[(size_t)v0 * NV * N + i] = x;
	}
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* sa = base + e * PER_E;
	double* sb = sa + NV * N;
	double* sc = sb + NV * N;
	tp_apply<D, Q, NV>(sa, sb, sc, TO_GL ? sops->B : sops->Binv, node, active);
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			const size_t o = ((size_t)(v0 + e) * NV + k) * N + node;
			out[o] = sb[k * N + node];
			if (out_copy)
				out_copy[o] = sb[k * N + node];
		}
}

}  // namespace dgpu
