// Flux physics for the explicit DG residual, FP64, as device inline functions.
//
// Each function states the reference routine it computes. The GB300 FP64 pipe (2 DFMA per cycle per SM) is the
// binding resource, so the numerical fluxes are written to need as few FP64 instructions as the same
// mathematics allows: each side's state is reduced once (one reciprocal of the density), the normal flux is
// formed from the normal velocity instead of contracting the full physical flux with the normal, and
// divisions by the same quantity are replaced by one reciprocal. These regroupings change rounding only.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "dgpu_dual.cuh"

namespace dgpu {

using ::fabs;
using ::pow;
using ::sqrt;

constexpr double kGamma = 1.4;          // definitions_physics.h:23
constexpr double kGm1 = 0.4;            // definitions_physics.h:24
constexpr double kEpsPhys = 1.0e-13;    // definitions_physics.h:30
constexpr double kEps = 1.0e-15;        // definitions_tol.h:23

enum Pde { kAdvection = 1, kEuler = 3, kNavierStokes = 4 };
enum Viscosity { kViscosityConstant = 101, kViscositySutherland = 102 };   // definitions_physics.h:34-36
enum NumFlux { kUpwind = 11, kRoePike = 31, kLaxFriedrichs = 32 };

// min_abs_real_T / max_abs_real_T (general/math_functions_T.c:222-236); T = double, or Dual for Jacobians.
template <typename T>
__device__ __forceinline__ T min_abs_real(const T& a, const T& b)
{
	T c = (fabs(a) < fabs(b) ? a : b);
	return (c < 0.0 ? -c : c);
}
template <typename T>
__device__ __forceinline__ T max_abs_real(const T& a, const T& b)
{
	T c = (fabs(a) > fabs(b) ? a : b);
	return (c < 0.0 ? -c : c);
}

// Contravariant volume flux at one cubature node for the Euler equations:
//   fr_j[eq] = sum_i g[j*D+i] f_i[eq]
// with f the physical flux of compute_Flux_T_euler / compute_Flux_euler_0 (flux_euler_T.c:71-143, 259-298)
// and g the metric terms (pre-multiplied by the cubature weight) of constructor_flux_ref_piece_T
// (compute_rlhs_T.c:71-110). The contraction is regrouped through the contravariant momentum
// M_j = sum_i g[j*D+i] m_i (the mass flux fr_j[0] itself) and velocity U_j = M_j / rho, and the pressure takes
// rho |u|^2 as |m|^2 / rho: the same sums with fewer FP64 operations.
template <int D, typename T = double>
__device__ __forceinline__ void euler_flux_ref(const T* W, const double* g, T (*fr)[D + 2])
{
	const T rho = W[0], E = W[D + 1];
	const T rho_inv = 1.0 / rho;
	T m2 = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k)
		m2 += W[1 + k] * W[1 + k];
	const T p = kGm1 * (E - 0.5 * (m2 * rho_inv));
	const T Ep = E + p;
#pragma unroll
	for (int j = 0; j < D; ++j) {
		T M = 0.0;
#pragma unroll
		for (int i = 0; i < D; ++i)
			M += g[j * D + i] * W[1 + i];
		const T U = M * rho_inv;
		fr[j][0] = M;
#pragma unroll
		for (int m = 0; m < D; ++m)
			fr[j][1 + m] = W[1 + m] * U + p * g[j * D + m];
		fr[j][D + 1] = Ep * U;
	}
}

// One side of a face node for Lax-Friedrichs: m.n, the normal velocity Vn = m.n / rho, the pressure and the wave
// speed |V| + c, with rho |V|^2 formed as |m|^2 / rho (one reciprocal of the density, no velocity vector).
template <int D, typename T>
__device__ __forceinline__ void euler_side_lf(const T* W, const double* n, T& mn, T& Vn, T& p, T& lam)
{
	const T rho_inv = 1.0 / W[0];
	T m2 = 0.0;
	mn = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k) {
		m2 += W[1 + k] * W[1 + k];
		mn += n[k] * W[1 + k];
	}
	const T q = m2 * rho_inv;   // rho |V|^2
	Vn = mn * rho_inv;
	p = kGm1 * (W[D + 1] - 0.5 * q);
	lam = sqrt(q * rho_inv) + sqrt(kGamma * p * rho_inv);
}

// Lax-Friedrichs (compute_Numerical_Flux_T_euler_lax_friedrichs, numerical_flux_euler_T.c:60-327):
//   nF = 1/2 [ n.(F_L + F_R) + max(|V_L| + c_L, |V_R| + c_R) (W_L - W_R) ] x scale
// with n.F = (m.n, m Vn + p n, (E + p) Vn) of each side (compute_Flux_euler_0 contracted with n); the two sides'
// pressure terms share one product with n. scale (the face node's w J, or 1) is folded into the factor 1/2, which
// gives the same bits as scaling afterwards (the factor 1/2 is exact).
template <int D, typename T = double>
__device__ __forceinline__ void num_flux_lax_friedrichs(const T* WL, const T* WR, const double* n, T* nF,
                                                        double scale = 1.0)
{
	T mnL, VnL, pL, lamL, mnR, VnR, pR, lamR;
	euler_side_lf<D>(WL, n, mnL, VnL, pL, lamL);
	euler_side_lf<D>(WR, n, mnR, VnR, pR, lamR);
	const T maxV = (lamL > lamR ? lamL : lamR);
	const double h = 0.5 * scale;
	const T pLR = pL + pR;
	nF[0] = h * ((mnL + mnR) + maxV * (WL[0] - WR[0]));
#pragma unroll
	for (int k = 0; k < D; ++k)
		nF[1 + k] = h * ((WL[1 + k] * VnL + WR[1 + k] * VnR + pLR * n[k]) + maxV * (WL[1 + k] - WR[1 + k]));
	nF[D + 1] = h * (((WL[D + 1] + pL) * VnL + (WR[D + 1] + pR) * VnR) + maxV * (WL[D + 1] - WR[D + 1]));
}

// Roe-Pike with the entropy fix of Qu et al. 2015 (compute_Numerical_Flux_T_euler_roe_pike,
// numerical_flux_euler_T.c:470-778).
template <int D, typename T = double>
__device__ __forceinline__ void num_flux_roe_pike(const T* WL, const T* WR, const double* n, T* nF)
{
	const T rhoL = WL[0], rhoR = WR[0], EL = WL[D + 1], ER = WR[D + 1];
	const T rhoL_inv = 1.0 / rhoL, rhoR_inv = 1.0 / rhoR;
	T uL[D], uR[D];
	T V2L = 0.0, V2R = 0.0, VnL = 0.0, VnR = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k) {
		uL[k] = WL[1 + k] * rhoL_inv;
		uR[k] = WR[1 + k] * rhoR_inv;
		V2L += uL[k] * uL[k];
		V2R += uR[k] * uR[k];
		VnL += n[k] * uL[k];
		VnR += n[k] * uR[k];
	}
	const T pL = kGm1 * (EL - 0.5 * rhoL * V2L), HL = (EL + pL) * rhoL_inv;
	const T pR = kGm1 * (ER - 0.5 * rhoR * V2R), HR = (ER + pR) * rhoR_inv;

	// Roe averages (divisions by r + 1 through one reciprocal)
	const T r = sqrt(rhoR * rhoL_inv), rP1_inv = 1.0 / (r + 1.0), rho = r * rhoL;
	T u[D];
	T Vn = 0.0, V2 = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k) {
		u[k] = (r * uR[k] + uL[k]) * rP1_inv;
		Vn += n[k] * u[k];
		V2 += u[k] * u[k];
	}
	const T H = (r * HR + HL) * rP1_inv, c2 = kGm1 * (H - 0.5 * V2), c = sqrt(c2), c_inv = 1.0 / c;

	const T l1 = min_abs_real(VnL - c, Vn - c), l5 = max_abs_real(VnR + c, Vn + c);
	const T l234 = (Vn > 0.0 ? Vn : -Vn);

	const T drho = rhoR - rhoL, dE = ER - EL, dp = pR - pL, dVn = VnR - VnL;
	const T lc1 = 0.5 * (l5 + l1) - l234, lc2 = 0.5 * (l5 - l1);
	const T disInter1 = (lc1 * dp * c_inv + lc2 * rho * dVn) * c_inv;
	const T disInter2 = lc1 * rho * dVn + lc2 * dp * c_inv;

	const T rhoVnL = rhoL * VnL, rhoVnR = rhoR * VnR, pLR = pL + pR;
	nF[0] = 0.5 * ((rhoVnL + rhoVnR) - (l234 * drho + disInter1));
#pragma unroll
	for (int k = 0; k < D; ++k) {
		const T drhou = WR[1 + k] - WL[1 + k];
		const T nFk = rhoVnL * uL[k] + rhoVnR * uR[k] + n[k] * pLR;
		const T disk = l234 * drhou + disInter1 * u[k] + disInter2 * n[k];
		nF[1 + k] = 0.5 * (nFk - disk);
	}
	nF[D + 1] = 0.5 * ((VnL * (EL + pL) + VnR * (ER + pR)) - (l234 * dE + disInter1 * H + disInter2 * Vn));
}

// Upwind advection flux (compute_Numerical_Flux_T_advection_upwind, numerical_flux_advection_T.c:39-75).
template <int D>
__device__ __forceinline__ double num_flux_upwind(double uL, double uR, const double* n, const double* b)
{
	double b_dot_n = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k)
		b_dot_n += b[k] * n[k];
	return (b_dot_n > kEps ? b_dot_n * uL : b_dot_n * uR);
}

// ---- boundary values ----------------------------------------------------------------------------------------------
// BC codes after taking them modulo BC_STEP_SC (definitions_bc.h:33-64); set_function_pointers_num_flux_bc_advection
// and _euler (face_solver_T.c:203-275) select the boundary value by these.
constexpr int kBcStepSC = 10000;
enum BcCode {
	kBcRiemann = 101, kBcSlipWall = 102, kBcBackPressure = 103, kBcTotalTP = 104, kBcSupersonicIn = 105,
	kBcSupersonicOut = 106, kBcNoSlipAdiabatic = 111, kBcNoSlipDiabatic = 112, kBcNoSlipAllRotating = 113
};

// BC_Data (boundary_euler_T.c:44-49): the scalars the reference reads from the test case's input file.
struct BcData {
	double p_back;   // BC_BACKPRESSURE
	double t_total;  // BC_TOTAL_TP: total temperature, total pressure, specific gas constant
	double p_total;
	double r_s;
};

// True for the advection codes that take the upwind boundary value (inflow 1-3, outflow 11-13, upwind 41-46).
__host__ __device__ __forceinline__ bool bc_is_advection_upwind(int bc)
{
	return (bc >= 1 && bc <= 3) || (bc >= 11 && bc <= 13) || (bc >= 41 && bc <= 46);
}
__host__ __device__ __forceinline__ bool bc_is_euler(int bc)
{
	return bc >= kBcRiemann && bc <= kBcSupersonicOut;
}
// The boundary values the reference's Navier-Stokes takes (face_solver_T.c:277-300).
__host__ __device__ __forceinline__ bool bc_is_navier_stokes(int bc)
{
	return bc == kBcRiemann || bc == kBcSupersonicIn || bc == kBcSupersonicOut || bc == kBcNoSlipAdiabatic ||
	       bc == kBcNoSlipDiabatic || bc == kBcNoSlipAllRotating;
}

// Exterior state WR of an Euler boundary face node from the interior trace WL, the test case's solution at the node
// (ext, conserved: constructor_sol_bv) and the unit normal n (outward from the interior volume). bc is already
// reduced modulo kBcStepSC and is one of the four codes (the context validates them on creation).
//   kBcRiemann       constructor_Boundary_Value_T_euler_riemann (boundary_euler_T.c:99-180): the outgoing
//                    invariant Vn + 2c/(gamma-1) of the interior and the incoming one of the exterior give the
//                    normal velocity and speed of sound; entropy and tangential velocity come from the upwind side;
//                    supersonic faces take the upwind state whole;
//   kBcSlipWall      ..._euler_slipwall (:494-533): density and energy kept, momentum mirrored about the face;
//   kBcSupersonicIn  ..._euler_supersonic_inflow (:657-692): the exterior state;
//   kBcSupersonicOut ..._euler_supersonic_outflow (:705-745): the interior state;
//   kBcBackPressure  ..._euler_back_pressure (:772-866): the interior state where |V| >= c, else the interior
//                    velocity at pressure p_back and density gamma p_back / c^2;
//   kBcTotalTP       ..._euler_total_tp (:991-1120): the speed of sound from the interior's outgoing invariant and
//                    total enthalpy (the larger root of a quadratic), flow along the normal, temperature and
//                    pressure from the total values by the isentropic relations, density by the gas law.
template <int D, typename T>
__device__ __forceinline__ void euler_boundary_state(int bc, const T* WL, const double* ext, const double* n, T* WR,
                                                     const BcData& bd)
{
	constexpr int NV = D + 2;
	if (bc == kBcBackPressure || bc == kBcTotalTP) {
		const T rho_l = WL[0], rho_l_inv = 1.0 / rho_l;
		T u_l[D], V2_l = 0.0, Vn_l = 0.0;
#pragma unroll
		for (int k = 0; k < D; ++k) {
			u_l[k] = WL[1 + k] * rho_l_inv;
			V2_l += u_l[k] * u_l[k];
			Vn_l += n[k] * u_l[k];
		}
		const T p_l = kGm1 * (WL[D + 1] - 0.5 * rho_l * V2_l);
		const T c2_l = kGamma * p_l * rho_l_inv;
		if (bc == kBcBackPressure) {
			if (!(sqrt(V2_l) < sqrt(c2_l))) {
#pragma unroll
				for (int k = 0; k < NV; ++k)
					WR[k] = WL[k];
			} else {
				const T rho_b = (kGamma * bd.p_back) / c2_l;
				WR[0] = rho_b;
#pragma unroll
				for (int k = 0; k < D; ++k)
					WR[1 + k] = u_l[k] * rho_b;
				WR[D + 1] = bd.p_back * (1.0 / kGm1) + 0.5 * rho_b * V2_l;
			}
			return;
		}
		const T H_l = (WL[D + 1] + p_l) * rho_l_inv;
		const T R_l = Vn_l + (2.0 / kGm1) * sqrt(c2_l);
		constexpr double aQ = 1.0 + 2.0 / kGm1;
		const T bQ = -2.0 * R_l, cQ = 0.5 * kGm1 * (R_l * R_l - 2.0 * H_l);
		const T t1 = bQ * (-0.5 / aQ), t2 = sqrt(bQ * bQ - 4.0 * aQ * cQ) * (0.5 / aQ);
		const T cM = t1 - t2, cP = t1 + t2;
		const T c = (cM > cP ? cM : cP);
		const T Vn = R_l - (2.0 / kGm1) * c;
		const T M = Vn / c;
		const T Tb = bd.t_total / (1.0 + 0.5 * kGm1 * M * M);
		const T p = bd.p_total * pow(Tb * (1.0 / bd.t_total), kGamma / kGm1);
		const T rho = p / (bd.r_s * Tb);
		T V2 = 0.0;
		WR[0] = rho;
#pragma unroll
		for (int k = 0; k < D; ++k) {
			const T uk = Vn * n[k];
			V2 += uk * uk;
			WR[1 + k] = rho * uk;
		}
		WR[D + 1] = p * (1.0 / kGm1) + 0.5 * rho * V2;
		return;
	}
	if (bc == kBcSlipWall) {
		T rhoVn = 0.0;
#pragma unroll
		for (int k = 0; k < D; ++k)
			rhoVn += n[k] * WL[1 + k];
		WR[0] = WL[0];
#pragma unroll
		for (int k = 0; k < D; ++k)
			WR[1 + k] = WL[1 + k] - 2.0 * rhoVn * n[k];
		WR[D + 1] = WL[D + 1];
		return;
	}
	if (bc == kBcSupersonicIn) {
#pragma unroll
		for (int k = 0; k < NV; ++k)
			WR[k] = ext[k];
		return;
	}
	if (bc != kBcRiemann) {   // supersonic outflow
#pragma unroll
		for (int k = 0; k < NV; ++k)
			WR[k] = WL[k];
		return;
	}
	// Riemann: primitive variables of both sides
	const T rho_l = WL[0], rho_l_inv = 1.0 / rho_l;
	T u_l[D], V2_l = 0.0, Vn_l = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k) {
		u_l[k] = WL[1 + k] * rho_l_inv;
		V2_l += u_l[k] * u_l[k];
		Vn_l += n[k] * u_l[k];
	}
	const T p_l = kGm1 * (WL[D + 1] - 0.5 * rho_l * V2_l);
	const double rho_r = ext[0];
	double u_r[D], V2_r = 0.0, Vn_r = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k) {
		u_r[k] = ext[1 + k] / rho_r;
		V2_r += u_r[k] * u_r[k];
		Vn_r += n[k] * u_r[k];
	}
	const double p_r = kGm1 * (ext[D + 1] - 0.5 * rho_r * V2_r);
	const T c_l = sqrt(kGamma * p_l * rho_l_inv);
	const double c_r = ::sqrt(kGamma * p_r / rho_r);
	const T R_l = Vn_l + (2.0 / kGm1) * c_l;   // outgoing
	const T R_r = Vn_r - (2.0 / kGm1) * c_r;   // incoming
	const T Vn = 0.5 * (R_l + R_r), cc = 0.25 * kGm1 * (R_l - R_r);
	T rho, p, uvw[D];
	if (!(fabs(Vn) < fabs(cc))) {   // supersonic: the upwind side's state
		if (Vn < 0.0) {
			rho = rho_r;
			p = p_r;
#pragma unroll
			for (int k = 0; k < D; ++k)
				uvw[k] = u_r[k];
		} else {
			rho = rho_l;
			p = p_l;
#pragma unroll
			for (int k = 0; k < D; ++k)
				uvw[k] = u_l[k];
		}
	} else {                        // subsonic: entropy and tangential velocity from the upwind side
		const T c2g = (1.0 / kGamma) * cc * cc;
		if (Vn < 0.0) {
			const double s_r = p_r / ::pow(rho_r, kGamma);
			rho = pow(c2g / s_r, 1.0 / kGm1);
#pragma unroll
			for (int k = 0; k < D; ++k)
				uvw[k] = Vn * n[k] + (u_r[k] - Vn_r * n[k]);
		} else {
			const T s_l = p_l / pow(rho_l, kGamma);
			rho = pow(c2g / s_l, 1.0 / kGm1);
#pragma unroll
			for (int k = 0; k < D; ++k)
				uvw[k] = Vn * n[k] + (u_l[k] - Vn_l * n[k]);
		}
		p = c2g * rho;
	}
	T V2 = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k)
		V2 += uvw[k] * uvw[k];
	WR[0] = rho;
#pragma unroll
	for (int k = 0; k < D; ++k)
		WR[1 + k] = rho * uvw[k];
	WR[D + 1] = p * (1.0 / kGm1) + 0.5 * rho * V2;
}

// Exterior value of an advection boundary node (constructor_Boundary_Value_T_advection_upwind,
// boundary_advection_T.c:40-77): the exterior solution where b.n <= 0 (inflow), else the interior trace.
template <int D, typename T>
__device__ __forceinline__ T advection_boundary_value(const T& uL, double ext, const double* n, const double* b)
{
	double b_dot_n = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k)
		b_dot_n += b[k] * n[k];
	return b_dot_n <= 0.0 ? T(ext) : uL;
}

// ---- Navier-Stokes viscous flux -----------------------------------------------------------------------------------
// Viscous part of the Navier-Stokes flux at one node, subtracted from F[dir][eq] (the reference adds the negated
// viscous flux to the Euler flux: compute_Flux_12_T with compute_Flux_T_navier_stokes, flux_navier_stokes_T.c:175-284,
// 1005-1040). W: conserved state; G[dir][var]: its gradient. Velocity gradients (compute_duvw :708-720), stress
// tau = mu (grad u + grad u^T - 2/3 div u I) (compute_tau :776-799), scaled temperature gradient
// dTs = grad(E/rho) - 1/2 grad |u|^2 (compute_dTs :905-927), heat flux gamma/Pr mu dTs. mu: constant, or
// Sutherland's law mu = 0.08 mu_ref sqrt(T) / (1 + 112 / T), T = p / (rho r_s) (compute_mu_sutherland_T,
// solution_navier_stokes_T.c:246-256, solution_navier_stokes.h:31-32).
struct NsPhys {
	double mu, Pr, r_s;
	int viscosity;
	double wall_nf_E;   // BC_NOSLIP_DIABATIC: the wall's normal energy flux -mu Cp / Pr dTdn
};

template <int D, typename T>
__device__ __forceinline__ void ns_viscous_sub(const T* W, const T (*G)[D + 2], const NsPhys& ph, T (*F)[D + 2])
{
	const T rho = W[0], E = W[D + 1], rho_inv = 1.0 / rho;
	T u[D], du[D][D], V2 = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k) {
		u[k] = W[1 + k] * rho_inv;
		V2 += u[k] * u[k];
	}
#pragma unroll
	for (int s = 0; s < D; ++s)
#pragma unroll
		for (int x = 0; x < D; ++x)
			du[s][x] = rho_inv * (G[x][1 + s] - G[x][0] * u[s]);
	T mu = ph.mu;
	if (ph.viscosity == kViscositySutherland) {
		const T p = kGm1 * (E - 0.5 * rho * V2), Tt = p / (rho * ph.r_s);
		mu = 0.08 * ph.mu / (1.0 + 112.0 / Tt) * sqrt(Tt);
	}
	T div = 0.0;
#pragma unroll
	for (int k = 0; k < D; ++k)
		div += du[k][k];
	T tau[D][D];
#pragma unroll
	for (int a = 0; a < D; ++a)
#pragma unroll
		for (int b = 0; b < D; ++b)
			tau[a][b] = (a == b) ? mu * 2.0 * (du[a][a] - div * (1.0 / 3.0)) : mu * (du[b][a] + du[a][b]);
	const T kappa = (kGamma / ph.Pr) * mu;
#pragma unroll
	for (int x = 0; x < D; ++x) {
		const T dE_o_rho = rho_inv * rho_inv * (G[x][D + 1] * rho - E * G[x][0]);
		T dV2 = 0.0, ut = 0.0;
#pragma unroll
		for (int k = 0; k < D; ++k) {
			dV2 += 2.0 * u[k] * du[k][x];
			ut += u[k] * tau[x][k];
		}
		const T dTs = dE_o_rho - 0.5 * dV2;
#pragma unroll
		for (int k = 0; k < D; ++k)
			F[x][1 + k] = F[x][1 + k] - tau[k][x];
		F[x][D + 1] = F[x][D + 1] - (kappa * dTs + ut);
	}
}

}  // namespace dgpu
