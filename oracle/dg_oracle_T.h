/* Templated body of the CPU oracle; included twice by dg_oracle.c (Type = double, Type = double complex),
 * the way the reference compiles each *_T.c for 'd' and 'dc' (e.g.
 * src/simulation/solvers/dg/compute_volume_rlhs_dg.c:65-71).
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker, not the product.
 *
 * Required macros: Type, SUF(name) (name suffix), REAL_T(x), ABS_T(x), SQRT_T(x).
 */

/* Type min_abs_real_T / max_abs_real_T: src/general/math_functions_T.c:222-236. */
static Type SUF(min_abs_real)(const Type a, const Type b)
{
	Type c = (ABS_T(a) < ABS_T(b) ? a : b);
	if (REAL_T(c) < 0.0)
		c *= -1.0;
	return c;
}

static Type SUF(max_abs_real)(const Type a, const Type b)
{
	Type c = (ABS_T(a) > ABS_T(b) ? a : b);
	if (REAL_T(c) < 0.0)
		c *= -1.0;
	return c;
}

/* out (m x nc, column-major) += alpha * A (m x k, row-major) * B (k x nc, column-major).
 * The reference's mm_NNC_* products through cblas_dgemm (src/containers/matrix_math_T.c:178-201). */
static void SUF(mm_acc)(const int m, const int k, const int nc, const double alpha, const double* A,
                        const Type* B, Type* out)
{
	for (int c = 0; c < nc; ++c) {
		for (int i = 0; i < m; ++i) {
			Type s = 0.0;
			const double* a = &A[(size_t)i * k];
			const Type* b = &B[(size_t)k * c];
			for (int j = 0; j < k; ++j)
				s += a[j] * b[j];
			out[i + (size_t)m * c] += alpha * s;
		}
	}
}

/* Exterior ("right") state of a boundary face node from the interior state WL, the exterior state ext (the test
 * case's solution at the node, constructor_sol_bv) and the unit normal, by BC code (definitions_bc.h):
 *   BC_RIEMANN 101         constructor_Boundary_Value_T_euler_riemann        (boundary_euler_T.c:99-290)
 *   BC_SLIPWALL 102        constructor_Boundary_Value_T_euler_slipwall       (boundary_euler_T.c:494-545)
 *   BC_SUPERSONIC_IN 105   constructor_Boundary_Value_T_euler_supersonic_inflow  (:657-703)
 *   BC_SUPERSONIC_OUT 106  constructor_Boundary_Value_T_euler_supersonic_outflow (:705-770)
 *   BC_BACKPRESSURE 103    constructor_Boundary_Value_T_euler_back_pressure  (:772-866), p_back = bc_data[0]
 *   BC_TOTAL_TP 104        constructor_Boundary_Value_T_euler_total_tp       (:991-1120), bc_data[1..3] =
 *                          (t_total, p_total, r_s)
 *   advection (1-3, 11-13, 41-46)  constructor_Boundary_Value_T_advection_upwind (boundary_advection_T.c:40-95)
 * The code is taken modulo BC_STEP_SC = 10000 (straight/curved variants) as set_function_pointers_num_flux_bc_*
 * do (face_solver_T.c:203-275).
 * Returns 0, or -1 for a BC code this oracle does not provide. */
static int SUF(boundary_state)(const struct oracle_problem* P, const int bc, const Type* WL, const double* ext,
                               const double* n, Type* WR)
{
	const int d = P->d, nv = P->n_var;
	if (P->pde == ORACLE_PDE_ADVECTION) {
		/* every advection code (inflow 1-3, outflow 11-13, upwind 41-46) takes the upwind boundary value
		 * (set_function_pointers_num_flux_bc_advection, face_solver_T.c:203-226) */
		const int a = bc % 10000;
		if (!((a >= 1 && a <= 3) || (a >= 11 && a <= 13) || (a >= 41 && a <= 46)))
			return -1;
		double b_dot_n = 0.0;
		for (int k = 0; k < d; ++k)
			b_dot_n += P->b_adv[k] * n[k];
		WR[0] = (b_dot_n <= 0.0 ? (Type)ext[0] : WL[0]);   /* inflow: exterior; outflow: interior */
		return 0;
	}
	if (P->pde == ORACLE_PDE_NAVIER_STOKES) {
		/* set_function_pointers_num_flux_bc_navier_stokes (face_solver_T.c:277-300): Riemann and supersonic
		 * in/outflow as for Euler, and the no-slip walls. BC_NOSLIP_ADIABATIC 111 and BC_NOSLIP_DIABATIC 112
		 * (static wall, u_ex = 0): rho and E kept, momentum -rhouvw_l + 2 rho u_ex
		 * (constructor_Boundary_Value_T_navier_stokes_no_slip_flux_general, boundary_navier_stokes_T.c:258-304).
		 * BC_NOSLIP_ALL_ROTATING 113: every variable 2 s_ex - s_l, s_ex = (rho_b, rho_b u_ex, E_b) with the wall's
		 * velocity u_ex (compute_uvw_ex_rotating, omega about the z axis), which the caller supplies as the exterior
		 * state (constructor_Boundary_Value_T_navier_stokes_no_slip_all_general, :196-244). */
		const int b = bc % 10000;
		if (b == 111 || b == 112) {
			WR[0] = WL[0];
			for (int k = 0; k < d; ++k)
				WR[1 + k] = -WL[1 + k];
			WR[d + 1] = WL[d + 1];
			return 0;
		}
		if (b == 113) {
			for (int k = 0; k < nv; ++k)
				WR[k] = -WL[k] + 2.0 * ext[k];
			return 0;
		}
		if (b != 101 && b != 105 && b != 106)
			return -1;
	}
	switch (bc % 10000) {
	case 102: {   /* slip wall: rho and E kept, momentum reflected about the face */
		Type rhoVn = 0.0;
		for (int k = 0; k < d; ++k)
			rhoVn += n[k] * WL[1 + k];
		WR[0] = WL[0];
		for (int k = 0; k < d; ++k)
			WR[1 + k] = WL[1 + k] - 2.0 * rhoVn * n[k];
		WR[d + 1] = WL[d + 1];
		return 0;
	}
	case 105:
		for (int k = 0; k < nv; ++k)
			WR[k] = ext[k];
		return 0;
	case 103: {   /* back pressure: supersonic (|V| >= c) keeps the interior state, else p = p_back */
		const double p_back = P->bc_data[0];
		const Type rho_l = WL[0];
		Type u_l[3] = {0.0, 0.0, 0.0}, V2_l = 0.0;
		for (int k = 0; k < d; ++k) {
			u_l[k] = WL[1 + k] / rho_l;
			V2_l += u_l[k] * u_l[k];
		}
		const Type p_l = GM1 * (WL[d + 1] - 0.5 * rho_l * V2_l);
		const Type c2_l = GAMMA * p_l / rho_l;
		if (ABS_T(SQRT_T(V2_l)) >= ABS_T(SQRT_T(c2_l))) {
			for (int k = 0; k < nv; ++k)
				WR[k] = WL[k];
		} else {
			const Type rho_b = GAMMA * p_back / c2_l;
			WR[0] = rho_b;
			for (int k = 0; k < d; ++k)
				WR[1 + k] = u_l[k] * rho_b;
			WR[d + 1] = p_back / GM1 + 0.5 * rho_b * V2_l;
		}
		return 0;
	}
	case 104: {   /* total temperature and pressure: outgoing invariant + total enthalpy give c, flow along n */
		const double T_tot = P->bc_data[1], p_tot = P->bc_data[2], r_s = P->bc_data[3];
		const Type rho_l = WL[0];
		Type u_l[3] = {0.0, 0.0, 0.0}, V2_l = 0.0, Vn_l = 0.0;
		for (int k = 0; k < d; ++k) {
			u_l[k] = WL[1 + k] / rho_l;
			V2_l += u_l[k] * u_l[k];
			Vn_l += n[k] * u_l[k];
		}
		const Type p_l = GM1 * (WL[d + 1] - 0.5 * rho_l * V2_l);
		const Type c_l = SQRT_T(GAMMA * p_l / rho_l);
		const Type H_l = (WL[d + 1] + p_l) / rho_l;
		const Type R_l = Vn_l + 2.0 / GM1 * c_l;
		const double aQ = 1.0 + 2.0 / GM1;
		const Type bQ = -2.0 * R_l, cQ = 0.5 * GM1 * (R_l * R_l - 2.0 * H_l);
		const Type t1 = -bQ / (2.0 * aQ), t2 = SQRT_T(bQ * bQ - 4.0 * aQ * cQ) / (2.0 * aQ);
		const Type cM = t1 - t2, cP = t1 + t2;
		const Type c = (REAL_T(cM) > REAL_T(cP) ? cM : cP);
		const Type Vn = R_l - 2.0 / GM1 * c;
		const Type M = Vn / c;
		const Type T = T_tot / (1.0 + 0.5 * GM1 * M * M);
		const Type p = p_tot * POW_T(T / T_tot, GAMMA / GM1);
		const Type rho = p / (r_s * T);
		Type V2 = 0.0;
		for (int k = 0; k < d; ++k)
			V2 += (Vn * n[k]) * (Vn * n[k]);
		WR[0] = rho;
		for (int k = 0; k < d; ++k)
			WR[1 + k] = rho * (Vn * n[k]);
		WR[d + 1] = p / GM1 + 0.5 * rho * V2;
		return 0;
	}
	case 106:
		for (int k = 0; k < nv; ++k)
			WR[k] = WL[k];
		return 0;
	case 101: {
		/* primitive variables of both sides (convert_variables 'c' -> 'p') */
		const Type rho_l = WL[0];
		Type u_l[3] = {0.0, 0.0, 0.0}, V2_l = 0.0;
		for (int k = 0; k < d; ++k) {
			u_l[k] = WL[1 + k] / rho_l;
			V2_l += u_l[k] * u_l[k];
		}
		const Type p_l = GM1 * (WL[d + 1] - 0.5 * rho_l * V2_l);
		const double rho_r = ext[0];
		double u_r[3] = {0.0, 0.0, 0.0}, V2_r = 0.0;
		for (int k = 0; k < d; ++k) {
			u_r[k] = ext[1 + k] / rho_r;
			V2_r += u_r[k] * u_r[k];
		}
		const double p_r = GM1 * (ext[d + 1] - 0.5 * rho_r * V2_r);
		const Type c_l = SQRT_T(GAMMA * p_l / rho_l);
		const double c_r = sqrt(GAMMA * p_r / rho_r);
		Type Vn_l = 0.0;
		double Vn_r = 0.0;
		for (int k = 0; k < d; ++k) {
			Vn_l += n[k] * u_l[k];
			Vn_r += n[k] * u_r[k];
		}
		const Type R_l = Vn_l + 2.0 / GM1 * c_l;   /* outgoing Riemann invariant */
		const Type R_r = Vn_r - 2.0 / GM1 * c_r;   /* incoming */
		const Type Vn = 0.5 * (R_l + R_r), cc = 0.25 * GM1 * (R_l - R_r);
		Type rho, p, uvw[3] = {0.0, 0.0, 0.0};
		if (ABS_T(Vn) >= ABS_T(cc)) {   /* supersonic */
			if (REAL_T(Vn) < 0.0) {     /* inlet */
				rho = rho_r;
				for (int k = 0; k < d; ++k)
					uvw[k] = u_r[k];
				p = p_r;
			} else {                    /* outlet */
				rho = rho_l;
				for (int k = 0; k < d; ++k)
					uvw[k] = u_l[k];
				p = p_l;
			}
		} else {                        /* subsonic */
			Type uvw_t[3] = {0.0, 0.0, 0.0};
			if (REAL_T(Vn) < 0.0) {
				const double s_r = p_r / pow(rho_r, GAMMA);
				rho = POW_T(1.0 / GAMMA * cc * cc / s_r, 1.0 / GM1);
				for (int k = 0; k < d; ++k)
					uvw_t[k] = u_r[k] - Vn_r * n[k];
			} else {
				const Type s_l = p_l / POW_T(rho_l, GAMMA);
				rho = POW_T(1.0 / GAMMA * cc * cc / s_l, 1.0 / GM1);
				for (int k = 0; k < d; ++k)
					uvw_t[k] = u_l[k] - Vn_l * n[k];
			}
			for (int k = 0; k < d; ++k)
				uvw[k] = Vn * n[k] + uvw_t[k];
			p = 1.0 / GAMMA * cc * cc * rho;
		}
		/* back to conserved variables (convert_variables 'p' -> 'c') */
		Type V2 = 0.0;
		for (int k = 0; k < d; ++k)
			V2 += uvw[k] * uvw[k];
		WR[0] = rho;
		for (int k = 0; k < d; ++k)
			WR[1 + k] = rho * uvw[k];
		WR[d + 1] = p / GM1 + 0.5 * rho * V2;
		return 0;
	}
	default:
		return -1;
	}
}

/* Physical Euler flux at one node, f[dim + d*eq]: compute_Flux_T_euler + compute_Flux_euler_0
 * (src/simulation/test_case/flux/flux_euler_T.c:71-143, 259-298). */
static void SUF(flux_euler)(const int d, const Type* W, Type* f)
{
	const Type rho = W[0], E = W[d + 1];
	const Type rho_inv = 1.0 / rho;
	Type uvw[3] = {0.0, 0.0, 0.0}, V2 = 0.0;
	for (int k = 0; k < d; ++k) {
		uvw[k] = rho_inv * W[1 + k];
		V2 += uvw[k] * uvw[k];
	}
	const Type p = GM1 * (E - 0.5 * rho * V2);
	int ind = 0;
	for (int k = 0; k < d; ++k)
		f[ind++] = W[1 + k];
	for (int m = 0; m < d; ++m)
		for (int k = 0; k < d; ++k)
			f[ind++] = W[1 + m] * uvw[k] + (m == k ? p : 0.0);
	for (int k = 0; k < d; ++k)
		f[ind++] = (E + p) * uvw[k];
}

/* Viscous part of the Navier-Stokes flux at one node, subtracted from f[dim + d*eq] (the reference adds the negated
 * viscous flux to the Euler flux, compute_Flux_12_T with compute_Flux_T_navier_stokes, flux_navier_stokes_T.c:175-
 * 284, 1005-1040). W: conserved state; G[dx + d*var]: its gradient. Velocity gradients (compute_duvw :708-720),
 * stress tau = mu (grad u + grad u^T - 2/3 div u I) (compute_tau :776-799), scaled temperature gradient
 * dTs = grad(E/rho) - 1/2 grad |u|^2 (compute_dTs :905-927), heat flux gamma/Pr mu dTs; mu constant or Sutherland's
 * law mu = c1 sqrt(T) / (1 + c2 / T), c1 = 0.08 mu, c2 = 112, T = p / (rho r_s) (compute_mu_sutherland_T,
 * solution_navier_stokes_T.c:246-256, solution_navier_stokes.h:31-32). */
static void SUF(flux_ns_sub)(const struct oracle_problem* P, const Type* W, const Type* G, Type* f)
{
	const int d = P->d;
	const Type rho = W[0], E = W[d + 1], rho_inv = 1.0 / rho;
	Type u[3] = {0.0, 0.0, 0.0}, du[3][3], V2 = 0.0;
	for (int k = 0; k < d; ++k) {
		u[k] = W[1 + k] * rho_inv;
		V2 += u[k] * u[k];
	}
	for (int s = 0; s < d; ++s)
		for (int x = 0; x < d; ++x)
			du[s][x] = rho_inv * (G[x + d * (1 + s)] - G[x + d * 0] * u[s]);
	Type mu = P->mu;
	if (P->viscosity == ORACLE_VISCOSITY_SUTHERLAND) {
		const Type p = GM1 * (E - 0.5 * rho * V2), T = p / (rho * P->r_s);
		mu = 0.08 * P->mu / (1.0 + 112.0 / T) * SQRT_T(T);
	}
	Type div = 0.0;
	for (int k = 0; k < d; ++k)
		div += du[k][k];
	Type tau[3][3];
	for (int a = 0; a < d; ++a)
		for (int b = 0; b < d; ++b)
			tau[a][b] = (a == b) ? mu * 2.0 * (du[a][a] - div / 3.0) : mu * (du[b][a] + du[a][b]);
	for (int x = 0; x < d; ++x) {
		const Type dE_o_rho = rho_inv * rho_inv * (G[x + d * (d + 1)] * rho - E * G[x + d * 0]);
		Type dV2 = 0.0;
		for (int k = 0; k < d; ++k)
			dV2 += 2.0 * u[k] * du[k][x];
		const Type dTs = dE_o_rho - 0.5 * dV2;
		Type ut = 0.0;
		for (int k = 0; k < d; ++k)
			ut += u[k] * tau[x][k];
		for (int k = 0; k < d; ++k)
			f[x + d * (1 + k)] -= tau[k][x];
		f[x + d * (d + 1)] -= GAMMA / P->Pr * mu * dTs + ut;
	}
}

/* Lax-Friedrichs: numerical_flux_euler_T.c:60-327. WL/WR are per-node state vectors, n is the node's
 * unit normal; writes nF[eq]. */
static void SUF(num_flux_lf)(const int d, const Type* WL, const Type* WR, const double* n, Type* nF)
{
	const int neq = d + 2;
	Type VL, VR, cL, cR;
	{
		const Type rho = WL[0], rho_inv = 1.0 / rho;
		Type V2 = 0.0;
		for (int k = 0; k < d; ++k) {
			const Type u = WL[1 + k] * rho_inv;
			V2 += u * u;
		}
		VL = SQRT_T(V2);
		const Type p = GM1 * (WL[d + 1] - 0.5 * rho * V2);
		cL = SQRT_T(GAMMA * p / rho);
	}
	{
		const Type rho = WR[0], rho_inv = 1.0 / rho;
		Type V2 = 0.0;
		for (int k = 0; k < d; ++k) {
			const Type u = WR[1 + k] * rho_inv;
			V2 += u * u;
		}
		VR = SQRT_T(V2);
		const Type p = GM1 * (WR[d + 1] - 0.5 * rho * V2);
		cR = SQRT_T(GAMMA * p / rho);
	}
	const Type maxlL = VL + cL, maxlR = VR + cR;
	const Type maxV = (REAL_T(maxlL) > REAL_T(maxlR) ? maxlL : maxlR);
	Type FL[15], FR[15];
	SUF(flux_euler)(d, WL, FL);
	SUF(flux_euler)(d, WR, FR);
	for (int eq = 0; eq < neq; ++eq) {
		Type s = 0.0;
		for (int k = 0; k < d; ++k)
			s += n[k] * (FL[k + d * eq] + FR[k + d * eq]);
		nF[eq] = 0.5 * (s + maxV * (WL[eq] - WR[eq]));
	}
}

/* Roe-Pike with the entropy fix of Qu et al. (2015), numerical_flux_euler_T.c:470-778. */
static void SUF(num_flux_roe)(const int d, const Type* WL, const Type* WR, const double* n, Type* nF)
{
	const Type rhoL = WL[0], rhoR = WR[0], EL = WL[d + 1], ER = WR[d + 1];
	const Type rhoL_inv = 1.0 / rhoL, rhoR_inv = 1.0 / rhoR;
	Type uL[3] = {0, 0, 0}, uR[3] = {0, 0, 0};
	Type V2L = 0.0, V2R = 0.0, VnL = 0.0, VnR = 0.0;
	for (int k = 0; k < d; ++k) {
		uL[k] = WL[1 + k] * rhoL_inv;
		uR[k] = WR[1 + k] * rhoR_inv;
		V2L += uL[k] * uL[k];
		V2R += uR[k] * uR[k];
		VnL += n[k] * uL[k];
		VnR += n[k] * uR[k];
	}
	const Type pL = GM1 * (EL - 0.5 * rhoL * V2L), HL = (EL + pL) * rhoL_inv;
	const Type pR = GM1 * (ER - 0.5 * rhoR * V2R), HR = (ER + pR) * rhoR_inv;

	const Type r = SQRT_T(rhoR / rhoL), rP1 = r + 1.0, rho = r * rhoL;
	Type u[3] = {0, 0, 0}, Vn = 0.0, V2 = 0.0;
	for (int k = 0; k < d; ++k) {
		u[k] = (r * uR[k] + uL[k]) / rP1;
		Vn += n[k] * u[k];
		V2 += u[k] * u[k];
	}
	const Type H = (r * HR + HL) / rP1, c2 = GM1 * (H - 0.5 * V2), c = SQRT_T(c2);

	const Type l1 = SUF(min_abs_real)(VnL - c, Vn - c), l5 = SUF(max_abs_real)(VnR + c, Vn + c),
	           l234 = (REAL_T(Vn) > 0.0 ? Vn : -Vn);

	const Type drho = rhoR - rhoL, dE = ER - EL, dp = pR - pL, dVn = VnR - VnL;
	const Type lc1 = 0.5 * (l5 + l1) - l234, lc2 = 0.5 * (l5 - l1);
	const Type disInter1 = lc1 * dp / (c * c) + lc2 * rho * dVn / c, disInter2 = lc1 * rho * dVn + lc2 * dp / c;

	const Type rhoVnL = rhoL * VnL, rhoVnR = rhoR * VnR, pLR = pL + pR;
	nF[0] = 0.5 * ((rhoVnL + rhoVnR) - (l234 * drho + disInter1));
	for (int k = 0; k < d; ++k) {
		const Type drhou = rhoR * uR[k] - rhoL * uL[k];
		const Type nFk = rhoVnL * uL[k] + rhoVnR * uR[k] + n[k] * pLR;
		const Type disk = l234 * drhou + disInter1 * u[k] + disInter2 * n[k];
		nF[1 + k] = 0.5 * (nFk - disk);
	}
	nF[d + 1] = 0.5 * ((VnL * (EL + pL) + VnR * (ER + pR)) - (l234 * dE + disInter1 * H + disInter2 * Vn));
}

/* Explicit DG residual (before M^-1): compute_rlhs_common_dg (solve_dg.c:182-189) with
 * compute_volume_rlhs_dg (compute_volume_rlhs_dg_T.c:53-72 -> compute_volume_rlhs_T.c:145-177,
 * compute_rlhs_T.c:71-110) and compute_face_rlhs_dg (compute_face_rlhs_dg_T.c:88-114 ->
 * boundary_T.c:42-145, compute_face_rlhs_T.c:297-359). sol/rhs: per volume (n_vs x n_var) column-major. */
/* A boundary face (no right volume): the interior trace, the exterior state of its BC at every node, the numerical
 * flux with the interior normal, and the lift into the interior volume only (compute_face_rlhs_T.c:297-310 with
 * Solver_Face_T::constructor_Boundary_Value_fcl, face_solver_T.c:246-274). */
/* Navier-Stokes: the partially corrected gradient of the interior side (gv + eta gf of this face, cv0_vs_fc) is
 * also the boundary gradient (constructor_Boundary_Value_T_grad_from_internal; the no-slip walls copy the density and
 * momentum gradients, boundary_navier_stokes_T.c:306-352), the central viscous flux is added, and on a no-slip
 * adiabatic wall the total normal energy flux is set to nf_E = 0 (nf_E_provided, set_provided_Numerical_Flux_members,
 * numerical_flux_central_T.c:222-231; DIABATIC_FLUX_CONSTANT_ZERO), on a diabatic one to nf_E = -mu Cp / Pr dTdn
 * (DIABATIC_FLUX_CONSTANT). gv, gf: as ns_gradients writes them, else NULL. */
static int SUF(boundary_face)(const struct oracle_ctx* c, const int f, const Type* sol, Type* rhs, Type* sL, Type* nnf,
                              const Type* gv, const Type* gf)
{
	const struct oracle_problem* P = &c->P;
	const int d = P->d, nv = P->n_var, neq = P->n_var;
	const int vL = P->face_vol[2 * f], lfL = P->face_lf[2 * f];
	const struct oracle_face_ops* FL = &P->face_ops[P->face_ops_idx[2 * f]];
	const int n_fc = FL->n_fc;
	const double* nrm = &P->normals_fc[c->fc_off[f] * d];
	const double* jf = &P->jacobian_det_fc[c->fc_off[f]];
	const double* ext = &P->bc_state_fc[c->fc_off[f] * nv];
	for (size_t i = 0; i < (size_t)n_fc * nv; ++i)
		sL[i] = 0.0;
	SUF(mm_acc)(n_fc, FL->n_vs, nv, 1.0, &FL->cv0_vs_fc[(size_t)lfL * n_fc * FL->n_vs], &sol[c->state_off[vL]], sL);
	Type* gp = NULL;
	if (gv) {
		const size_t fstride = (size_t)c->max_vs * nv;
		gp = calloc((size_t)n_fc * nv * d, sizeof(Type));
		Type* tmp = malloc(sizeof(Type) * fstride);
		for (int dir = 0; dir < d; ++dir) {
			const Type* gfL = &gf[((size_t)(2 * f) * d + dir) * fstride];
			for (size_t i = 0; i < (size_t)FL->n_vs * nv; ++i)
				tmp[i] = gv[c->n_state * dir + c->state_off[vL] + i] + 1.01 * 2 * d * gfL[i];
			SUF(mm_acc)(n_fc, FL->n_vs, nv, 1.0, &FL->cv0_vs_fc[(size_t)lfL * n_fc * FL->n_vs], tmp,
			            &gp[(size_t)dir * n_fc * nv]);
		}
		free(tmp);
	}
	for (int i = 0; i < n_fc; ++i) {
		Type WL[5], WR[5], nF[5];
		for (int k = 0; k < nv; ++k)
			WL[k] = sL[i + (size_t)n_fc * k];
		const double* ni = &nrm[(size_t)i * d];
		if (SUF(boundary_state)(P, P->bc_fc[f], WL, &ext[(size_t)i * nv], ni, WR) != 0) {
			free(gp);
			return -1;
		}
		if (P->pde != ORACLE_PDE_ADVECTION) {
			if (P->num_flux == ORACLE_NUM_FLUX_ROE_PIKE)
				SUF(num_flux_roe)(d, WL, WR, ni, nF);
			else
				SUF(num_flux_lf)(d, WL, WR, ni, nF);
		} else {
			double b_dot_n = 0.0;
			for (int k = 0; k < d; ++k)
				b_dot_n += P->b_adv[k] * ni[k];
			nF[0] = (b_dot_n > ORACLE_EPS ? b_dot_n * WL[0] : b_dot_n * WR[0]);
		}
		if (gp) {
			Type G[15], FvL[15], FvR[15];
			for (int var = 0; var < nv; ++var)
				for (int x = 0; x < d; ++x)
					G[x + d * var] = gp[(size_t)x * n_fc * nv + i + (size_t)n_fc * var];
			for (int k = 0; k < d * neq; ++k)
				FvL[k] = FvR[k] = 0.0;
			SUF(flux_ns_sub)(P, WL, G, FvL);
			SUF(flux_ns_sub)(P, WR, G, FvR);
			for (int eq = 0; eq < neq; ++eq)
				for (int x = 0; x < d; ++x)
					nF[eq] += 0.5 * ni[x] * (FvL[x + d * eq] + FvR[x + d * eq]);
			if (P->bc_fc[f] % 10000 == 111)
				nF[d + 1] = 0.0;
			else if (P->bc_fc[f] % 10000 == 112)   /* -mu Cp / Pr dTdn, Cp = gamma / (gamma - 1) r_s */
				nF[d + 1] = -P->mu * (GAMMA / GM1 * P->r_s) / P->Pr * P->dTdn;
		}
		for (int k = 0; k < neq; ++k)
			nnf[i + (size_t)n_fc * k] = nF[k] * jf[i];
	}
	free(gp);
	SUF(mm_acc)(FL->n_vs, n_fc, neq, -1.0, &FL->tw0_vt_fc[(size_t)lfL * FL->n_vs * n_fc], nnf, &rhs[c->state_off[vL]]);
	return 0;
}

/* BR2 gradients of the Navier-Stokes residual (compute_grad_coef_dg_T, compute_grad_coef_dg_T.c:60-316) for the
 * explicit, non-collocated case:
 *   volume:  grad_coef_v[dir] = M^-1 tw0_vt_vc (sum_k m(., dir, k) cv1_vs_vc[k]) sol   (:168-214, 342-358);
 *   faces:   grad_coef_f[side][dir] = M^-1 tw0_vt_fc (J_f n_dir (s_num - s_side)), the central numerical
 *            solution s_num = (s_L + s_R) / 2 (get_sol_scale :674-686), side 1 in its own face-node order
 *            (:216-316, 424-440);
 *   total:   grad_coef = grad_coef_v + sum over the volume's faces of grad_coef_f (:503-525).
 * gv, gt: d x n_state ([dir][state]); gf: per face side (2f + s) d x (max_vs x n_var). */
static void SUF(ns_gradients)(const struct oracle_ctx* c, const Type* sol, Type* gv, Type* gf, Type* gt)
{
	const struct oracle_problem* P = &c->P;
	const int d = P->d, nv = P->n_var;
	const size_t ns = c->n_state, fstride = (size_t)c->max_vs * nv;
	Type* dr = malloc(sizeof(Type) * (size_t)c->max_vc * nv * d);
	Type* t = malloc(sizeof(Type) * (size_t)c->max_vc * nv);
	Type* y = malloc(sizeof(Type) * fstride);
	for (size_t i = 0; i < ns * d; ++i)
		gv[i] = gt[i] = 0.0;
	for (size_t i = 0; i < (size_t)P->n_faces * 2 * d * fstride; ++i)
		gf[i] = 0.0;
	for (int v = 0; v < P->n_volumes; ++v) {
		const struct oracle_group* G = &P->groups[P->vol_group[v]];
		const int n_vs = G->n_vs, n_vc = G->n_vc;
		const Type* s = &sol[c->state_off[v]];
		const double* m = &P->metrics_vc[c->vc_off[v] * d * d];
		for (size_t i = 0; i < (size_t)n_vc * nv * d; ++i)
			dr[i] = 0.0;
		for (int k = 0; k < d; ++k)
			SUF(mm_acc)(n_vc, n_vs, nv, 1.0, &G->cv1_vs_vc[(size_t)k * n_vc * n_vs], s, &dr[(size_t)k * n_vc * nv]);
		for (int dir = 0; dir < d; ++dir) {
			for (int var = 0; var < nv; ++var)
				for (int n = 0; n < n_vc; ++n) {
					Type a = 0.0;
					for (int k = 0; k < d; ++k)
						a += m[n + (size_t)n_vc * (dir + d * k)] * dr[(size_t)k * n_vc * nv + n + (size_t)n_vc * var];
					t[n + (size_t)n_vc * var] = G->w_vc[n] * a;   /* tw0_vt_vc = cv0^T diag(w_vc) */
				}
			for (int var = 0; var < nv; ++var)
				for (int i = 0; i < n_vs; ++i) {
					Type a = 0.0;
					for (int n = 0; n < n_vc; ++n)
						a += G->cv0_vs_vc[(size_t)n * n_vs + i] * t[n + (size_t)n_vc * var];
					y[i + (size_t)n_vs * var] = a;
				}
			SUF(mm_acc)(n_vs, n_vs, nv, 1.0, &c->m_inv[c->minv_off[v]], y, &gv[ns * dir + c->state_off[v]]);
		}
	}
	Type* sL = malloc(sizeof(Type) * (size_t)c->max_fc * nv);
	Type* sR0 = malloc(sizeof(Type) * (size_t)c->max_fc * nv);
	Type* X = malloc(sizeof(Type) * (size_t)c->max_fc * nv);
	Type* XR = malloc(sizeof(Type) * (size_t)c->max_fc * nv);
	for (int f = 0; f < P->n_faces; ++f) {
		const int vL = P->face_vol[2 * f], vR = P->face_vol[2 * f + 1];
		const int lfL = P->face_lf[2 * f], lfR = P->face_lf[2 * f + 1];
		const struct oracle_face_ops* FL = &P->face_ops[P->face_ops_idx[2 * f]];
		const struct oracle_face_ops* FR = &P->face_ops[P->face_ops_idx[2 * f + 1]];
		const int n_fc = FL->n_fc;
		const int* nc = &P->nc_fc[c->fc_off[f]];
		const double* nrm = &P->normals_fc[c->fc_off[f] * d];
		const double* jf = &P->jacobian_det_fc[c->fc_off[f]];
		if (vR < 0) {   /* boundary face: s_num = (s_L + s_b) / 2 with s_b its boundary value
		                 * (compute_g_coef_related_boundary, compute_grad_coef_dg_T.c:527-640) */
			const double* ext = &P->bc_state_fc[c->fc_off[f] * nv];
			for (size_t i = 0; i < (size_t)n_fc * nv; ++i)
				sL[i] = 0.0;
			SUF(mm_acc)(n_fc, FL->n_vs, nv, 1.0, &FL->cv0_vs_fc[(size_t)lfL * n_fc * FL->n_vs], &sol[c->state_off[vL]],
			            sL);
			for (int i = 0; i < n_fc; ++i) {
				Type WL[5], WB[5];
				for (int k = 0; k < nv; ++k)
					WL[k] = sL[i + (size_t)n_fc * k];
				SUF(boundary_state)(P, P->bc_fc[f], WL, &ext[(size_t)i * nv], &nrm[(size_t)i * d], WB);
				for (int k = 0; k < nv; ++k)
					sR0[i + (size_t)n_fc * k] = WB[k];
			}
			for (int dir = 0; dir < d; ++dir) {
				for (int var = 0; var < nv; ++var)
					for (int i = 0; i < n_fc; ++i) {
						const size_t o = i + (size_t)n_fc * var;
						X[o] = jf[i] * nrm[(size_t)i * d + dir] * 0.5 * (sR0[o] - sL[o]);
					}
				Type* gL = &gf[((size_t)(2 * f) * d + dir) * fstride];
				for (size_t i = 0; i < fstride; ++i)
					y[i] = 0.0;
				SUF(mm_acc)(FL->n_vs, n_fc, nv, 1.0, &FL->tw0_vt_fc[(size_t)lfL * FL->n_vs * n_fc], X, y);
				SUF(mm_acc)(FL->n_vs, FL->n_vs, nv, 1.0, &c->m_inv[c->minv_off[vL]], y, gL);
				for (size_t i = 0; i < (size_t)FL->n_vs * nv; ++i)
					gt[ns * dir + c->state_off[vL] + i] += gL[i];
			}
			continue;
		}
		for (size_t i = 0; i < (size_t)n_fc * nv; ++i)
			sL[i] = sR0[i] = 0.0;
		SUF(mm_acc)(n_fc, FL->n_vs, nv, 1.0, &FL->cv0_vs_fc[(size_t)lfL * n_fc * FL->n_vs], &sol[c->state_off[vL]], sL);
		SUF(mm_acc)(n_fc, FR->n_vs, nv, 1.0, &FR->cv0_vs_fc[(size_t)lfR * n_fc * FR->n_vs], &sol[c->state_off[vR]], sR0);
		for (int dir = 0; dir < d; ++dir) {
			for (int var = 0; var < nv; ++var)
				for (int i = 0; i < n_fc; ++i) {
					const size_t o = i + (size_t)n_fc * var;
					X[o] = jf[i] * nrm[(size_t)i * d + dir] * 0.5 * (sR0[nc[i] + (size_t)n_fc * var] - sL[o]);
					XR[nc[i] + (size_t)n_fc * var] = X[o];   /* side 1: J_f (-n) (s_num - s_R) = the same values */
				}
			Type* gL = &gf[((size_t)(2 * f) * d + dir) * fstride];
			Type* gR = &gf[((size_t)(2 * f + 1) * d + dir) * fstride];
			for (size_t i = 0; i < fstride; ++i)
				y[i] = 0.0;
			SUF(mm_acc)(FL->n_vs, n_fc, nv, 1.0, &FL->tw0_vt_fc[(size_t)lfL * FL->n_vs * n_fc], X, y);
			SUF(mm_acc)(FL->n_vs, FL->n_vs, nv, 1.0, &c->m_inv[c->minv_off[vL]], y, gL);
			for (size_t i = 0; i < fstride; ++i)
				y[i] = 0.0;
			SUF(mm_acc)(FR->n_vs, n_fc, nv, 1.0, &FR->tw0_vt_fc[(size_t)lfR * FR->n_vs * n_fc], XR, y);
			SUF(mm_acc)(FR->n_vs, FR->n_vs, nv, 1.0, &c->m_inv[c->minv_off[vR]], y, gR);
			for (size_t i = 0; i < (size_t)FL->n_vs * nv; ++i)
				gt[ns * dir + c->state_off[vL] + i] += gL[i];
			for (size_t i = 0; i < (size_t)FR->n_vs * nv; ++i)
				gt[ns * dir + c->state_off[vR] + i] += gR[i];
		}
	}
	for (size_t i = 0; i < ns * d; ++i)
		gt[i] += gv[i];
	free(dr); free(t); free(y); free(sL); free(sR0); free(X); free(XR);
}

/* remote: per face n_fc x n_var column-major (at fc_off[f] n_var), the trace of a side whose volume belongs to another
 * partition (face_vol == ORACLE_REMOTE_VOLUME), in that side's own face-node order; NULL when no side is remote. */
static int SUF(residual_raw)(const struct oracle_ctx* c, const Type* sol, Type* rhs, const double* remote)
{
	const struct oracle_problem* P = &c->P;
	const int d = P->d, nv = P->n_var, neq = P->n_var;

	for (size_t i = 0; i < c->n_state; ++i)
		rhs[i] = 0.0;

	Type* s_vc = malloc(sizeof(Type) * (size_t)c->max_vc * nv);
	Type* fr = malloc(sizeof(Type) * (size_t)c->max_vc * neq * d);
	Type* sL = malloc(sizeof(Type) * (size_t)c->max_fc * nv);
	Type* sR0 = malloc(sizeof(Type) * (size_t)c->max_fc * nv);
	Type* sR = malloc(sizeof(Type) * (size_t)c->max_fc * nv);
	Type* nnf = malloc(sizeof(Type) * (size_t)c->max_fc * neq);
	Type* nnfR = malloc(sizeof(Type) * (size_t)c->max_fc * neq);
	const int ns_pde = P->pde == ORACLE_PDE_NAVIER_STOKES;
	const size_t fstride = (size_t)c->max_vs * nv;
	Type *gv = NULL, *gf = NULL, *gt = NULL, *g_vc = NULL, *gpL = NULL, *gpR0 = NULL, *gpR = NULL, *tmp = NULL;
	if (ns_pde) {
		gv = malloc(sizeof(Type) * c->n_state * d);
		gt = malloc(sizeof(Type) * c->n_state * d);
		gf = malloc(sizeof(Type) * (size_t)(P->n_faces > 0 ? P->n_faces : 1) * 2 * d * fstride);
		g_vc = malloc(sizeof(Type) * (size_t)c->max_vc * nv * d);
		gpL = malloc(sizeof(Type) * (size_t)c->max_fc * nv * d);
		gpR0 = malloc(sizeof(Type) * (size_t)c->max_fc * nv * d);
		gpR = malloc(sizeof(Type) * (size_t)c->max_fc * nv * d);
		tmp = malloc(sizeof(Type) * fstride);
		SUF(ns_gradients)(c, sol, gv, gf, gt);
	}
	/* BR2's scaling of a face's own lifting in the face gradient: PENALTY_SCALING * NFMAX
	 * (compute_face_rlhs_dg_T.c:273-295, NFMAX = 2 DIM for the TP elements, definitions_elements.h:60-76) */
	const double eta = 1.01 * 2 * d;

	/* ---- volume term ---- */
	for (int v = 0; v < P->n_volumes; ++v) {
		const struct oracle_group* G = &P->groups[P->vol_group[v]];
		const int n_vs = G->n_vs, n_vc = G->n_vc;
		const Type* s = &sol[c->state_off[v]];
		Type* r = &rhs[c->state_off[v]];
		const double* m = &P->metrics_vc[c->vc_off[v] * d * d];
		for (size_t i = 0; i < (size_t)n_vc * nv; ++i)
			s_vc[i] = 0.0;
		SUF(mm_acc)(n_vc, n_vs, nv, 1.0, G->cv0_vs_vc, s, s_vc);
		if (ns_pde) {   /* the gradient at the cubature nodes: cv0_vr_vc grad_coef */
			for (size_t i = 0; i < (size_t)n_vc * nv * d; ++i)
				g_vc[i] = 0.0;
			for (int dir = 0; dir < d; ++dir)
				SUF(mm_acc)(n_vc, n_vs, nv, 1.0, G->cv0_vs_vc, &gt[c->n_state * dir + c->state_off[v]],
				            &g_vc[(size_t)dir * n_vc * nv]);
		}
		for (size_t i = 0; i < (size_t)n_vc * neq * d; ++i)
			fr[i] = 0.0;
		for (int n = 0; n < n_vc; ++n) {
			Type W[5], f[15];
			for (int k = 0; k < nv; ++k)
				W[k] = s_vc[n + (size_t)n_vc * k];
			if (P->pde != ORACLE_PDE_ADVECTION) {
				SUF(flux_euler)(d, W, f);
				if (ns_pde) {
					Type Gn[15];
					for (int var = 0; var < nv; ++var)
						for (int x = 0; x < d; ++x)
							Gn[x + d * var] = g_vc[(size_t)x * n_vc * nv + n + (size_t)n_vc * var];
					SUF(flux_ns_sub)(P, W, Gn, f);
				}
			} else {
				for (int k = 0; k < d; ++k)
					f[k] = P->b_adv[k] * W[0];
			}
			/* fr(n,eq,dim0) = sum_dim1 m(n,dim1,dim0) f(n,dim1,eq)  (compute_rlhs_T.c:71-110) */
			for (int eq = 0; eq < neq; ++eq)
				for (int d0 = 0; d0 < d; ++d0)
					for (int d1 = 0; d1 < d; ++d1)
						fr[n + (size_t)n_vc * (eq + (size_t)neq * d0)] +=
							m[n + (size_t)n_vc * (d1 + d * d0)] * f[d1 + d * eq];
		}
		/* rhs += sum_dim tw1_vt_vc[dim] . fr(:,:,dim)  (compute_volume_rlhs_T.c:166-177) */
		for (int dim = 0; dim < d; ++dim)
			SUF(mm_acc)(n_vs, n_vc, neq, 1.0, &G->tw1_vt_vc[(size_t)dim * n_vs * n_vc],
			            &fr[(size_t)n_vc * neq * dim], r);
		/* rhs += tw0_vt_vc (J_vc s), tw0_vt_vc = cv0_vs_vc^T diag(w_vc) (compute_source_rhs_dg_like,
		 * compute_rlhs.c:47-57; solution_advection_default_T.c:79-94) */
		if (P->source_vc) {
			const double* sv = &P->source_vc[c->vc_off[v] * nv];
			const double* J = &P->jacobian_det_vc[c->vc_off[v]];
			for (int k = 0; k < neq; ++k)
				for (int i = 0; i < n_vs; ++i) {
					double acc = 0.0;
					for (int n = 0; n < n_vc; ++n)
						acc += G->cv0_vs_vc[(size_t)n * n_vs + i] * (G->w_vc[n] * (J[n] * sv[n + (size_t)n_vc * k]));
					r[i + (size_t)n_vs * k] += acc;
				}
		}
	}

	/* ---- face term ---- */
	for (int f = 0; f < P->n_faces; ++f) {
		const int vL = P->face_vol[2 * f], vR = P->face_vol[2 * f + 1];
		const int remL = (vL == ORACLE_REMOTE_VOLUME), remR = (vR == ORACLE_REMOTE_VOLUME);
		if ((remL || remR) && (!remote || ns_pde)) {
			free(s_vc); free(fr); free(sL); free(sR0); free(sR); free(nnf); free(nnfR);
			free(gv); free(gf); free(gt); free(g_vc); free(gpL); free(gpR0); free(gpR); free(tmp);
			return ORACLE_ERR_ARG;
		}
		if (vR < 0 && !remR) {
			if (SUF(boundary_face)(c, f, sol, rhs, sL, nnf, gv, gf) != 0) {
				free(s_vc); free(fr); free(sL); free(sR0); free(sR); free(nnf); free(nnfR);
				free(gv); free(gf); free(gt); free(g_vc); free(gpL); free(gpR0); free(gpR); free(tmp);
				return ORACLE_ERR_ARG;
			}
			continue;
		}
		const int lfL = P->face_lf[2 * f], lfR = P->face_lf[2 * f + 1];
		const struct oracle_face_ops* FL = &P->face_ops[P->face_ops_idx[2 * f]];
		const struct oracle_face_ops* FR = &P->face_ops[P->face_ops_idx[2 * f + 1]];
		const int n_fc = FL->n_fc;
		const int* nc = &P->nc_fc[c->fc_off[f]];
		const double* nrm = &P->normals_fc[c->fc_off[f] * d];
		const double* jf = &P->jacobian_det_fc[c->fc_off[f]];
		for (size_t i = 0; i < (size_t)n_fc * nv; ++i)
			sL[i] = sR0[i] = 0.0;
		if (remL)
			for (size_t i = 0; i < (size_t)n_fc * nv; ++i)
				sL[i] = remote[c->fc_off[f] * nv + i];
		else
			SUF(mm_acc)(n_fc, FL->n_vs, nv, 1.0, &FL->cv0_vs_fc[(size_t)lfL * n_fc * FL->n_vs], &sol[c->state_off[vL]], sL);
		if (remR)
			for (size_t i = 0; i < (size_t)n_fc * nv; ++i)
				sR0[i] = remote[c->fc_off[f] * nv + i];
		else
			SUF(mm_acc)(n_fc, FR->n_vs, nv, 1.0, &FR->cv0_vs_fc[(size_t)lfR * n_fc * FR->n_vs], &sol[c->state_off[vR]], sR0);
		/* right trace reordered to the left's face-node order (boundary_T.c:80-92) */
		for (int k = 0; k < nv; ++k)
			for (int i = 0; i < n_fc; ++i)
				sR[i + (size_t)n_fc * k] = sR0[nc[i] + (size_t)n_fc * k];
		if (ns_pde) {
			/* each side's partially corrected gradient at the face nodes: cv0_vr_fc (grad_coef_v + eta
			 * grad_coef_f of this face) (constructor_partial_grad_fc_interp, compute_face_rlhs_dg_T.c:239-262),
			 * the right side's in the left's node order */
			for (size_t i = 0; i < (size_t)n_fc * nv * d; ++i)
				gpL[i] = gpR0[i] = 0.0;
			for (int dir = 0; dir < d; ++dir) {
				const Type* gfL = &gf[((size_t)(2 * f) * d + dir) * fstride];
				const Type* gfR = &gf[((size_t)(2 * f + 1) * d + dir) * fstride];
				for (size_t i = 0; i < (size_t)FL->n_vs * nv; ++i)
					tmp[i] = gv[c->n_state * dir + c->state_off[vL] + i] + eta * gfL[i];
				SUF(mm_acc)(n_fc, FL->n_vs, nv, 1.0, &FL->cv0_vs_fc[(size_t)lfL * n_fc * FL->n_vs], tmp,
				            &gpL[(size_t)dir * n_fc * nv]);
				for (size_t i = 0; i < (size_t)FR->n_vs * nv; ++i)
					tmp[i] = gv[c->n_state * dir + c->state_off[vR] + i] + eta * gfR[i];
				SUF(mm_acc)(n_fc, FR->n_vs, nv, 1.0, &FR->cv0_vs_fc[(size_t)lfR * n_fc * FR->n_vs], tmp,
				            &gpR0[(size_t)dir * n_fc * nv]);
				for (int k = 0; k < nv; ++k)
					for (int i = 0; i < n_fc; ++i)
						gpR[(size_t)dir * n_fc * nv + i + (size_t)n_fc * k] =
							gpR0[(size_t)dir * n_fc * nv + nc[i] + (size_t)n_fc * k];
			}
		}
		for (int i = 0; i < n_fc; ++i) {
			Type WL[5], WR[5], nF[5];
			for (int k = 0; k < nv; ++k) {
				WL[k] = sL[i + (size_t)n_fc * k];
				WR[k] = sR[i + (size_t)n_fc * k];
			}
			const double* ni = &nrm[(size_t)i * d];
			if (P->pde != ORACLE_PDE_ADVECTION) {
				if (P->num_flux == ORACLE_NUM_FLUX_ROE_PIKE)
					SUF(num_flux_roe)(d, WL, WR, ni, nF);
				else
					SUF(num_flux_lf)(d, WL, WR, ni, nF);
			} else {
				/* numerical_flux_advection_T.c:39-75 */
				double b_dot_n = 0.0;
				for (int k = 0; k < d; ++k)
					b_dot_n += P->b_adv[k] * ni[k];
				nF[0] = (b_dot_n > ORACLE_EPS ? b_dot_n * WL[0] : b_dot_n * WR[0]);
			}
			if (ns_pde) {   /* + the central viscous flux (compute_Numerical_Flux_T_central, numerical_flux_central_T.c) */
				Type GL[15], GR[15], fL[15], fR[15];
				for (int var = 0; var < nv; ++var)
					for (int x = 0; x < d; ++x) {
						GL[x + d * var] = gpL[(size_t)x * n_fc * nv + i + (size_t)n_fc * var];
						GR[x + d * var] = gpR[(size_t)x * n_fc * nv + i + (size_t)n_fc * var];
					}
				for (int k = 0; k < d * neq; ++k)
					fL[k] = fR[k] = 0.0;
				SUF(flux_ns_sub)(P, WL, GL, fL);
				SUF(flux_ns_sub)(P, WR, GR, fR);
				for (int eq = 0; eq < neq; ++eq)
					for (int x = 0; x < d; ++x)
						nF[eq] += 0.5 * ni[x] * (fL[x + d * eq] + fR[x + d * eq]);
			}
			/* scale_by_Jacobian_e_T (compute_face_rlhs_T.c:337-342) */
			for (int k = 0; k < neq; ++k)
				nnf[i + (size_t)n_fc * k] = nF[k] * jf[i];
		}
		/* rhs_L -= tw0_vt_fc[L] nnf ; rhs_R -= tw0_vt_fc[R] (-nnf in the right's node order)
		 * (compute_face_rlhs_T.c:297-310, 347-359). The right side is brought back to its own face-node
		 * order with the inverse of the trace permutation; the reference applies nc_fc itself, which is the
		 * same whenever nc_fc is an involution. */
		if (!remL)
			SUF(mm_acc)(FL->n_vs, n_fc, neq, -1.0, &FL->tw0_vt_fc[(size_t)lfL * FL->n_vs * n_fc], nnf, &rhs[c->state_off[vL]]);
		for (int k = 0; k < neq; ++k)
			for (int i = 0; i < n_fc; ++i)
				nnfR[nc[i] + (size_t)n_fc * k] = -nnf[i + (size_t)n_fc * k];
		if (!remR)
			SUF(mm_acc)(FR->n_vs, n_fc, neq, -1.0, &FR->tw0_vt_fc[(size_t)lfR * FR->n_vs * n_fc], nnfR, &rhs[c->state_off[vR]]);
	}

	free(s_vc); free(fr); free(sL); free(sR0); free(sR); free(nnf); free(nnfR);
	free(gv); free(gf); free(gt); free(g_vc); free(gpL); free(gpR0); free(gpR); free(tmp);
	return ORACLE_OK;
}

/* rhs <- M^-1 rhs per volume: scale_rhs_by_m_inv_std (solve_dg.c:265-272). */
static void SUF(scale_m_inv)(const struct oracle_ctx* c, Type* rhs)
{
	const struct oracle_problem* P = &c->P;
	const int nv = P->n_var;
	Type* tmp = malloc(sizeof(Type) * (size_t)c->max_vs * nv);
	for (int v = 0; v < P->n_volumes; ++v) {
		const int n_vs = P->groups[P->vol_group[v]].n_vs;
		Type* r = &rhs[c->state_off[v]];
		for (size_t i = 0; i < (size_t)n_vs * nv; ++i)
			tmp[i] = 0.0;
		SUF(mm_acc)(n_vs, n_vs, nv, 1.0, &c->m_inv[c->minv_off[v]], r, tmp);
		for (size_t i = 0; i < (size_t)n_vs * nv; ++i)
			r[i] = tmp[i];
	}
	free(tmp);
}
