// Navier-Stokes residual on the TP path: the Euler flux plus the viscous flux, with the BR2 gradients of the
// reference's explicit DG solver (compute_grad_coef_dg_T, src/simulation/solvers/dg/compute_grad_coef_dg_T.c:60-316;
// constructor_partial_grad_fc_interp, compute_face_rlhs_dg_T.c:239-295) in GL nodal space.
//
// In GL space with the GLL basis and the GL cubature of the same size, V (GLL -> GL) is square and invertible, so the
// reference's operators reduce as follows (M = V^T diag(w J) V, E = GL -> face interpolation along the normal):
//   grad_coef_v = M^-1 tw0_vt_vc (sum_k m(., dir, k) cv1_vs_vc[k]) u  ->  V grad_coef_v = (1/J) sum_k m(dir, k) d_r_k u_gl,
//       the physical gradient of the solution at the GL nodes (d_r_k: GL collocation derivative);
//   grad_coef_f = M^-1 tw0_vt_fc (J_f n (s_num - s))                 ->  diag(1/(w J)) E^T X,
//       X = w_f J_f n (s_R - s_L) / 2 at the face nodes (the same values seen from either side);
//   cv0_vr_fc grad_coef_f (the face's own lifting at its nodes)      ->  lambda X, lambda(t) = sum_m lb[m]^2 / (w J)(t, m):
//       diagonal in the face nodes because E^T puts a face node's value on one line of volume nodes.
// Per stage: tp_ns_grad_kernel (the volume gradient, kept, and the state and gradient traces), tp_ns_face_kernel (X,
// the partial face gradients g_tr + eta lambda X, Roe-Pike / Lax-Friedrichs plus the central viscous flux),
// tp_ns_volume_kernel (the kept gradient + the lifting of X from every face, the Euler and viscous contravariant flux,
// Dgl^T contraction), then the ordinary lift kernel. All three are bound by the FP64 issue rate, so the volume
// kernel reads the gradient (D NV doubles a node) rather than forming it again (about D (NV Q + NV D) FMAs a node).
#pragma once

#include <type_traits>

#include "dgpu_tp.cuh"

namespace dgpu {

// Start index and stride of the line of volume nodes under face node t of local face lf (normal direction nd).
template <int D, int Q>
__device__ __forceinline__ void face_line(int nd, int t, int* base, int* stride)
{
	const int t0 = (D == 2 ? t : t % Q), t1 = (D == 2 ? 0 : t / Q);
	if (D == 2) {
		*stride = (nd == 0 ? 1 : Q);
		*base = (nd == 0 ? t0 * Q : t0);
	} else {
		*stride = (nd == 0 ? 1 : (nd == 1 ? Q : Q * Q));
		*base = (nd == 0 ? t0 * Q + t1 * Q * Q : (nd == 1 ? t0 + t1 * Q * Q : t0 + t1 * Q));
	}
}

// Face node index of volume node `node` on a face with normal direction nd (tangential directions ascending).
template <int D, int Q>
__device__ __forceinline__ int face_node_of(int node, int nd)
{
	const int c0 = node_coord<Q>(node, 0), c1 = node_coord<Q>(node, 1), c2 = (D == 3 ? node_coord<Q>(node, 2) : 0);
	if (D == 2)
		return nd == 0 ? c1 : c0;
	return nd == 0 ? c1 + Q * c2 : (nd == 1 ? c0 + Q * c2 : c0 + Q * c1);
}

// lambda(t) of every face side at its own nodes (setup).
template <int D, int Q>
__global__ void __launch_bounds__(256) tp_ns_lambda_kernel(const TPOps ops, const TPParams P, double* lam)
{
	using S = TPShape<D, Q>;
	constexpr int NF = S::NF, N = S::N;
	const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= (long long)P.n_vol * 2 * D * NF)
		return;
	const int v = (int)(gid / (2 * D * NF)), r = (int)(gid % (2 * D * NF));
	const int lf = r / NF, t = r % NF, nd = lf >> 1, side = lf & 1;
	int base, stride;
	face_line<D, Q>(nd, t, &base, &stride);
	double s = 0.0;
	for (int m = 0; m < Q; ++m) {
		const double l = ops.lb[side][m];
		s += l * l * P.inv_wJ[(size_t)v * N + base + m * stride];
	}
	lam[(size_t)P.vol_face[(size_t)v * 2 * D + lf] * NF + t] = s;
}

// Shared memory per element of the two NS element kernels (doubles): the state and D gradient components.
template <int D, int Q, int NV>
struct NsSmem {
	static constexpr int PER_E = (1 + D) * NV * TPShape<D, Q>::N;
};

// GL values of the element into su (from GLL coefficients when GLL_IN), the GL collocation derivatives into sd and
// the physical volume gradient at this thread's node into g. All threads call it (it synchronises).
template <int D, int Q, int NV, bool GLL_IN>
__device__ __forceinline__ void ns_element_gradient(const TPOps* sops, const TPParams& P, int v, int node, bool active,
                                                    double* su, double* sd, double (*g)[NV])
{
	constexpr int N = TPShape<D, Q>::N;
	if (GLL_IN) {
		tp_apply<D, Q, NV>(su, sd, sd + NV * N, sops->B, node, active);
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				su[k * N + node] = sd[k * N + node];
		__syncthreads();
	}
	if (active)
#pragma unroll
		for (int k = 0; k < D; ++k)
			tp_pass<D, Q, NV>(su, sd + k * NV * N, sops->Dgl, k, node);
	__syncthreads();
	if (active) {
		const double iwJ = P.inv_wJ[(size_t)v * N + node];
		double gm[D * D];
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			gm[c] = P.gmet[((size_t)v * D * D + c) * N + node];
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
}

template <int D, int Q, int NV, bool GLL_IN>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_ns_grad_kernel(const TPOps ops, const TPParams P, const double* __restrict__ u)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF, E = S::E, PER_E = NsSmem<D, Q, NV>::PER_E;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	load_ops(sops, ops);
	const int tid = threadIdx.x, v0 = blockIdx.x * E, n_here = min(E, P.n_vol - v0);
	for (int i = tid; i < n_here * NV * N; i += blockDim.x)
		base[(i / (NV * N)) * PER_E + i % (NV * N)] = u[(size_t)v0 * NV * N + i];
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* su = base + e * PER_E;
	double* sd = su + NV * N;
	const int v = v0 + e;
	double g[D][NV];
	ns_element_gradient<D, Q, NV, GLL_IN>(sops, P, v, node, active, su, sd, g);
	if (active)
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int var = 0; var < NV; ++var) {
				sd[(dir * NV + var) * N + node] = g[dir][var];
				P.ns_gv[(((size_t)v * D + dir) * NV + var) * N + node] = g[dir][var];
			}
	__syncthreads();
	if (!active)
		return;
	// traces of the state and of the volume gradient on the 2D local faces
	for (int it = node; it < 2 * D * NF; it += N) {
		const int lf = it / NF, t = it % NF, nd = lf >> 1, side = lf & 1;
		int b, stride;
		face_line<D, Q>(nd, t, &b, &stride);
		const int fs = P.vol_face[(size_t)v * 2 * D + lf];
		double* ds = P.traces + (size_t)fs * NV * NF;
		double* dg = P.ns_gtr + (size_t)fs * D * NV * NF;
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			double s = 0.0;
#pragma unroll
			for (int m = 0; m < Q; ++m)
				s += sops->lb[side][m] * su[k * N + b + m * stride];
			ds[k * NF + t] = s;
		}
		for (int c = 0; c < D * NV; ++c) {
			double s = 0.0;
#pragma unroll
			for (int m = 0; m < Q; ++m)
				s += sops->lb[side][m] * sd[c * N + b + m * stride];
			dg[c * NF + t] = s;
		}
	}
}

// The contravariant Euler minus viscous flux at a volume node: fr_j = sum_i w J dr_j/dx_i (f_i(W) - f_v,i(W, G))
// (compute_volume_rlhs_T.c:71-110 with the Navier-Stokes flux of flux_navier_stokes_T.c), gm the weighted metric terms.
template <int D, typename T>
__device__ __forceinline__ void ns_flux_ref(const T* W, const T (*G)[D + 2], const double* gm, const NsPhys& ns,
                                            T (*fr)[D + 2])
{
	constexpr int NV = D + 2;
	euler_flux_ref<D>(W, gm, fr);
	T Fv[D][NV];
#pragma unroll
	for (int i = 0; i < D; ++i)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			Fv[i][k] = T(0.0);
	ns_viscous_sub<D, T>(W, G, ns, Fv);
#pragma unroll
	for (int j = 0; j < D; ++j)
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			T a = T(0.0);
#pragma unroll
			for (int i = 0; i < D; ++i)
				a = a + gm[j * D + i] * Fv[i][k];
			fr[j][k] = fr[j][k] + a;
		}
}

// Scalar helpers of the face and volume bodies below: T = double (the residual) or Dual<1> (the residual and its
// directional derivative, the tangent quantities read from and written to a second parameter set Pd).
__device__ __forceinline__ void ns_set(double& x, double v, double) { x = v; }
__device__ __forceinline__ void ns_set(Dual<1>& x, double v, double d)
{
	x.v = v;
	x.d[0] = d;
}
__device__ __forceinline__ double ns_val(const double& x) { return x; }
__device__ __forceinline__ double ns_val(const Dual<1>& x) { return x.v; }
__device__ __forceinline__ double ns_der(const double&) { return 0.0; }
__device__ __forceinline__ double ns_der(const Dual<1>& x) { return x.d[0]; }

// The Navier-Stokes boundary value WR of a face node from the interior trace WL (set_function_pointers_num_flux_bc_
// navier_stokes, face_solver_T.c:277-300): Riemann and supersonic in/outflow as for Euler; the static no-slip walls
// keep rho and E and mirror the momentum (boundary_navier_stokes_T.c:258-304); the rotating wall takes 2 s_ex - s_l
// for every variable, s_ex = (rho_b, rho_b u_wall, E_b) given as the exterior state (:196-244). ext: the node's
// exterior state, its variables ext_stride apart.
template <int D, typename T>
__device__ __forceinline__ void ns_boundary_state(int code, const T* WL, const double* ext, int ext_stride,
                                                  const double* n, const BcData& bcd, T* WR)
{
	constexpr int NV = D + 2;
	if (code == kBcNoSlipAdiabatic || code == kBcNoSlipDiabatic) {
		WR[0] = WL[0];
#pragma unroll
		for (int k = 0; k < D; ++k)
			WR[1 + k] = -WL[1 + k];
		WR[D + 1] = WL[D + 1];
	} else if (code == kBcNoSlipAllRotating) {
#pragma unroll
		for (int k = 0; k < NV; ++k)
			WR[k] = 2.0 * ext[k * ext_stride] - WL[k];
	} else {
		double e[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			e[k] = ext[k * ext_stride];
		euler_boundary_state<D, T>(code, WL, e, n, WR, bcd);
	}
}

// The face-node function on scalar type T (double, or dual numbers for the linearisations): from the left trace WL,
// the right trace WR (a boundary face, code >= 0, forms it from WL instead, as its BC), the gradient traces GtL, GtR
// (GtR unused on a boundary face), it gives X = w_f J_f n (W_R - W_L) / 2 and the face flux
// o = w_f J_f (F*(W_L, W_R) + n . (F_v(W_L, G_L) + F_v(W_R, G_R)) / 2) with the partial face gradients
// G_s = Gt_s + eta lambda_s X. code: the face's BC code, or -1 inside; ext: its exterior state at the node.
template <int D, int FLUX, typename T>
__device__ __forceinline__ void ns_face_flux(int code, const double* ext, int ext_stride, const BcData& bcd,
                                             const NsPhys& ph, double eta, const double* n, double sc, double lamL,
                                             double lamR, const T* WL, T* WR, const T (*GtL)[D + 2],
                                             const T (*GtR)[D + 2], T (*X)[D + 2], T* o)
{
	constexpr int NV = D + 2;
	const bool bnd = code >= 0;
	if (bnd)
		ns_boundary_state<D, T>(code, WL, ext, ext_stride, n, bcd, WR);
	T GL[D][NV], GR[D][NV];
#pragma unroll
	for (int dir = 0; dir < D; ++dir)
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			X[dir][k] = (0.5 * sc * n[dir]) * (WR[k] - WL[k]);
			GL[dir][k] = GtL[dir][k] + (eta * lamL) * X[dir][k];
			// on a boundary face the exterior gradient is the interior one (grad_from_internal; the walls copy it)
			GR[dir][k] = !bnd ? GtR[dir][k] + (eta * lamR) * X[dir][k] : GL[dir][k];
		}
	T nF[NV];
	if constexpr (FLUX == kRoePike)
		num_flux_roe_pike<D, T>(WL, WR, n, nF);
	else
		num_flux_lax_friedrichs<D, T>(WL, WR, n, nF);
	T FL[D][NV], FR[D][NV];
#pragma unroll
	for (int dir = 0; dir < D; ++dir)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			FL[dir][k] = FR[dir][k] = T(0.0);
	ns_viscous_sub<D, T>(WL, GL, ph, FL);
	ns_viscous_sub<D, T>(WR, GR, ph, FR);
#pragma unroll
	for (int k = 0; k < NV; ++k) {
		T s = T(0.0);
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
			s = s + n[dir] * (FL[dir][k] + FR[dir][k]);
		// a static wall sets the total normal energy flux to nf_E: 0 when adiabatic, -mu Cp / Pr dTdn when
		// diabatic (set_provided_Numerical_Flux_members, numerical_flux_central_T.c:222-231)
		const bool wall_E = (k == D + 1 && (code == kBcNoSlipAdiabatic || code == kBcNoSlipDiabatic));
		const double nf_E = code == kBcNoSlipDiabatic ? ph.wall_nf_E * sc : 0.0;
		o[k] = wall_E ? T(nf_E) : (nF[k] + 0.5 * s) * sc;
	}
}

// ns_face_flux with the uniform context's boundary list: b is the face's index in it, or -1.
template <int D, int FLUX, typename T>
__device__ __forceinline__ void ns_face_core(const TPParams& P, int b, int t, int NF, const double* n, double sc,
                                             double lamL, double lamR, const T* WL, T* WR, const T (*GtL)[D + 2],
                                             const T (*GtR)[D + 2], T (*X)[D + 2], T* o)
{
	const int code = b >= 0 ? P.bc_code[b] : -1;
	const double* ext = b >= 0 ? P.bc_ext + (size_t)b * (D + 2) * NF + t : nullptr;
	ns_face_flux<D, FLUX, T>(code, ext, NF, P.bc_data, P.ns, P.ns_eta, n, sc, lamL, lamR, WL, WR, GtL, GtR, X, o);
}

// One face node of the residual (T = double) or of the residual and its directional derivative (T = Dual<1>, the
// tangent traces, gradient traces and outputs in Pd): loads the traces, runs ns_face_core, stores X and the flux.
template <int D, int Q, int FLUX, typename T>
__device__ __forceinline__ void ns_face_node(const TPParams& P, const TPParams& Pd, int f, int t)
{
	constexpr int NF = TPShape<D, Q>::NF, NV = D + 2;
	constexpr bool TAN = !std::is_same<T, double>::value;
	const int b = P.bnd ? P.bnd[f] : -1;   // boundary face: its index in the boundary list
	const int tR = (b < 0 && P.nc) ? P.nc[(size_t)f * NF + t] : t;
	const double* fg = P.fgeo + (size_t)f * (D + 1) * NF;
	double n[D];
	T WL[NV], WR[NV];
#pragma unroll
	for (int k = 0; k < D; ++k)
		n[k] = fg[k * NF + t];
	const double sc = fg[D * NF + t];
	const size_t oL = (size_t)(2 * f) * NV * NF, oR = (size_t)(2 * f + 1) * NV * NF;
#pragma unroll
	for (int k = 0; k < NV; ++k)
		ns_set(WL[k], P.traces[oL + k * NF + t], TAN ? Pd.traces[oL + k * NF + t] : 0.0);
	if (b < 0)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			ns_set(WR[k], P.traces[oR + k * NF + tR], TAN ? Pd.traces[oR + k * NF + tR] : 0.0);
	const double lamL = P.ns_lam[(size_t)(2 * f) * NF + t];
	const double lamR = b < 0 ? P.ns_lam[(size_t)(2 * f + 1) * NF + tR] : lamL;
	const size_t gL = (size_t)(2 * f) * D * NV * NF, gR = (size_t)(2 * f + 1) * D * NV * NF;
	T GtL[D][NV], GtR[D][NV];
#pragma unroll
	for (int dir = 0; dir < D; ++dir)
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			const size_t cl = gL + (dir * NV + k) * NF + t;
			ns_set(GtL[dir][k], P.ns_gtr[cl], TAN ? Pd.ns_gtr[cl] : 0.0);
			if (b < 0) {
				const size_t cr = gR + (dir * NV + k) * NF + tR;
				ns_set(GtR[dir][k], P.ns_gtr[cr], TAN ? Pd.ns_gtr[cr] : 0.0);
			}
		}
	T X[D][NV], o[NV];
	ns_face_core<D, FLUX, T>(P, b, t, NF, n, sc, lamL, lamR, WL, WR, GtL, GtR, X, o);
#pragma unroll
	for (int dir = 0; dir < D; ++dir)
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			const size_t ox = ((size_t)f * D * NV + dir * NV + k) * NF + t;
			P.ns_X[ox] = ns_val(X[dir][k]);
			if (TAN)
				Pd.ns_X[ox] = ns_der(X[dir][k]);
		}
	const size_t on = (size_t)f * NV * NF + t;
#pragma unroll
	for (int k = 0; k < NV; ++k) {
		P.nnf[on + k * NF] = ns_val(o[k]);
		if (TAN)
			Pd.nnf[on + k * NF] = ns_der(o[k]);
	}
}

template <int D, int Q, int FLUX>
__global__ void __launch_bounds__(128) tp_ns_face_kernel(const TPParams P)
{
	constexpr int NF = TPShape<D, Q>::NF;
	const int gid = blockIdx.x * blockDim.x + threadIdx.x;
	if (gid < P.n_face * NF)
		ns_face_node<D, Q, FLUX, double>(P, P, gid / NF, gid % NF);
}

// The face kernel on dual numbers: primal outputs to P, tangent outputs to Pd (forward-mode linearisation).
template <int D, int Q, int FLUX>
__global__ void __launch_bounds__(128) tp_ns_jvp_face_kernel(const TPParams P, const TPParams Pd)
{
	constexpr int NF = TPShape<D, Q>::NF;
	const int gid = blockIdx.x * blockDim.x + threadIdx.x;
	if (gid < P.n_face * NF)
		ns_face_node<D, Q, FLUX, Dual<1>>(P, Pd, gid / NF, gid % NF);
}

template <int D, int Q, int NV, bool GLL_IN>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_ns_volume_kernel(const TPOps ops, const TPParams P, const double* __restrict__ u)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF, E = S::E, PER_E = NsSmem<D, Q, NV>::PER_E;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	load_ops(sops, ops);
	const int tid = threadIdx.x, v0 = blockIdx.x * E, n_here = min(E, P.n_vol - v0);
	for (int i = tid; i < n_here * NV * N; i += blockDim.x)
		base[(i / (NV * N)) * PER_E + i % (NV * N)] = u[(size_t)v0 * NV * N + i];
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* su = base + e * PER_E;
	double* sf = su + NV * N;
	const int v = v0 + e;
	if (GLL_IN) {   // GL values of the state
		tp_apply<D, Q, NV>(su, sf, sf + NV * N, sops->B, node, active);
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				su[k * N + node] = sf[k * N + node];
		__syncthreads();
	}
	double g[D][NV];
	if (active)
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int var = 0; var < NV; ++var)
				g[dir][var] = P.ns_gv[(((size_t)v * D + dir) * NV + var) * N + node];
	double fr[D][NV];
	if (active) {
		// + the lifting of every face's X (BR2 total gradient): inv_wJ lb[side][m] X at this node
		const double iwJ = P.inv_wJ[(size_t)v * N + node];
#pragma unroll
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int nd = lf >> 1, side = lf & 1;
			const int tf = face_node_of<D, Q>(node, nd);
			const int fs = P.vol_face[(size_t)v * 2 * D + lf], f = fs >> 1;
			const int tX = ((fs & 1) && P.nc_inv) ? P.nc_inv[(size_t)f * NF + tf] : tf;
			const double c = iwJ * sops->lb[side][node_coord<Q>(node, nd)];
			const double* X = P.ns_X + (size_t)f * D * NV * NF + tX;
#pragma unroll
			for (int dir = 0; dir < D; ++dir)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					g[dir][k] += c * X[(dir * NV + k) * NF];
		}
		double W[NV], gm[D * D];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			W[k] = su[k * N + node];
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			gm[c] = P.gmet[((size_t)v * D * D + c) * N + node];
		ns_flux_ref<D, double>(W, g, gm, P.ns, fr);
	}
	__syncthreads();   // everyone is done with sf's derivatives
	if (active)
#pragma unroll
		for (int j = 0; j < D; ++j)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				sf[(j * NV + k) * N + node] = fr[j][k];
	__syncthreads();
	if (!active)
		return;
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
			const double w = sops->Dgl[m][a];
#pragma unroll
			for (int k = 0; k < NV; ++k)
				acc[k] += w * sf[(j * NV + k) * N + b0 + m * stride];
		}
	}
#pragma unroll
	for (int k = 0; k < NV; ++k)
		P.vol_gl[((size_t)v * NV + k) * N + node] = acc[k];
}

// Volume term on dual numbers (forward-mode linearisation): the state and its direction from GLL coefficients u, du;
// the kept gradients (P.ns_gv, Pd.ns_gv) plus the liftings of X and its tangent; the Euler and viscous contravariant
// flux on Dual<1>; the Dgl^T contraction of the value into P.vol_gl, then of the derivative into Pd.vol_gl.
template <int D, int Q, int NV>
struct NsJvpSmem {
	static constexpr int PER_E = (2 + D) * NV * TPShape<D, Q>::N;   // su, sud, sf (also V's temporaries)
};

template <int D, int Q, int NV>
__global__ void __launch_bounds__(TPShape<D, Q>::THREADS)
tp_ns_jvp_volume_kernel(const TPOps ops, const TPParams P, const TPParams Pd, const double* __restrict__ u,
                        const double* __restrict__ du)
{
	using S = TPShape<D, Q>;
	constexpr int N = S::N, NF = S::NF, E = S::E, PER_E = NsJvpSmem<D, Q, NV>::PER_E;
	extern __shared__ double smem[];
	TPOps* sops = reinterpret_cast<TPOps*>(smem);
	double* base = smem + sizeof(TPOps) / 8;
	load_ops(sops, ops);
	const int tid = threadIdx.x, v0 = blockIdx.x * E, n_here = min(E, P.n_vol - v0);
	for (int i = tid; i < n_here * NV * N; i += blockDim.x) {
		const int e = i / (NV * N), r = i % (NV * N);
		base[e * PER_E + r] = u[(size_t)v0 * NV * N + i];
		base[e * PER_E + NV * N + r] = du[(size_t)v0 * NV * N + i];
	}
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* su = base + e * PER_E;
	double* sud = su + NV * N;
	double* sf = sud + NV * N;
	tp_apply<D, Q, NV>(su, sf, sf + NV * N, sops->B, node, active);
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			su[k * N + node] = sf[k * N + node];
	__syncthreads();
	tp_apply<D, Q, NV>(sud, sf, sf + NV * N, sops->B, node, active);
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			sud[k * N + node] = sf[k * N + node];
	__syncthreads();
	const int v = v0 + e;
	Dual<1> fr[D][NV];
	if (active) {
		Dual<1> g[D][NV], W[NV];
#pragma unroll
		for (int dir = 0; dir < D; ++dir)
#pragma unroll
			for (int var = 0; var < NV; ++var) {
				const size_t o = (((size_t)v * D + dir) * NV + var) * N + node;
				ns_set(g[dir][var], P.ns_gv[o], Pd.ns_gv[o]);
			}
		const double iwJ = P.inv_wJ[(size_t)v * N + node];
#pragma unroll
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int nd = lf >> 1, side = lf & 1;
			const int tf = face_node_of<D, Q>(node, nd);
			const int fs = P.vol_face[(size_t)v * 2 * D + lf], f = fs >> 1;
			const int tX = ((fs & 1) && P.nc_inv) ? P.nc_inv[(size_t)f * NF + tf] : tf;
			const double c = iwJ * sops->lb[side][node_coord<Q>(node, nd)];
			const size_t ox = (size_t)f * D * NV * NF + tX;
#pragma unroll
			for (int dir = 0; dir < D; ++dir)
#pragma unroll
				for (int k = 0; k < NV; ++k) {
					g[dir][k].v += c * P.ns_X[ox + (dir * NV + k) * NF];
					g[dir][k].d[0] += c * Pd.ns_X[ox + (dir * NV + k) * NF];
				}
		}
#pragma unroll
		for (int k = 0; k < NV; ++k)
			ns_set(W[k], su[k * N + node], sud[k * N + node]);
		double gm[D * D];
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			gm[c] = P.gmet[((size_t)v * D * D + c) * N + node];
		euler_flux_ref<D, Dual<1>>(W, gm, fr);
		Dual<1> Fv[D][NV];
#pragma unroll
		for (int i = 0; i < D; ++i)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				Fv[i][k] = Dual<1>(0.0);
		ns_viscous_sub<D, Dual<1>>(W, g, P.ns, Fv);
#pragma unroll
		for (int j = 0; j < D; ++j)
#pragma unroll
			for (int k = 0; k < NV; ++k)
#pragma unroll
				for (int i = 0; i < D; ++i)
					fr[j][k] = fr[j][k] + gm[j * D + i] * Fv[i][k];
	}
	// contraction of the value, then of the derivative, through the same shared buffer
	for (int pass = 0; pass < 2; ++pass) {
		__syncthreads();
		if (active)
#pragma unroll
			for (int j = 0; j < D; ++j)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					sf[(j * NV + k) * N + node] = pass == 0 ? fr[j][k].v : fr[j][k].d[0];
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
					const double w = sops->Dgl[m][a];
#pragma unroll
					for (int k = 0; k < NV; ++k)
						acc[k] += w * sf[(j * NV + k) * N + b0 + m * stride];
				}
			}
			double* out = pass == 0 ? P.vol_gl : Pd.vol_gl;
#pragma unroll
			for (int k = 0; k < NV; ++k)
				out[((size_t)v * NV + k) * N + node] = acc[k];
		}
	}
}

}  // namespace dgpu
