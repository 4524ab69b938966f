// Batched explicit DG residual over a mesh of several (element type, p) groups (QUAD or HEX, p = 1..4 mixed).
//
// Elements are stored group by group. A face between volumes of orders p_L and p_R is integrated with the face
// cubature of order p_f = max(p_L, p_R) (the reference's face order, face_solver.c:123-132): each volume
// writes its trace at the face's q_f = p_f + 1 GL points (tangential interpolation from its own q GL points when
// q_f > q), the face kernel evaluates the numerical flux there, and each volume applies the transpose of that
// interpolation before its lift. With q_f = q this reduces to the single-order kernels of dgpu_tp.cuh.
//
// Every kernel body is a __device__ function of (D, Q, ...) with a runtime number of elements per CTA, called
// either by one kernel launch per group ("plain per-group" form) or by one persistent kernel that walks a tile
// list covering all groups and dispatches on each tile's Q ("fused" form).
#pragma once

#include "dgpu_tp.cuh"

namespace dgpu {

constexpr int kMaxLf = 6;       // element-face slots per volume in elf (HEX has the most faces)
constexpr int kMaxOrd = 8;      // face orientations (QUAD faces)

struct BatchOps {
	TPOps t;
	double Iup[kQMax + 1][kQMax][kQMax];   // Iup[qf][i][a]: GL(q) Lagrange a at GL(qf) node i, qf >= q
};
static_assert(sizeof(BatchOps) % 8 == 0, "BatchOps is copied to shared memory as doubles");

struct BGroup {
	int q, n_vol, E;          // order+1, volumes, elements per CTA of the per-group form
	int first_tile;           // first tile of this group in the fused tile list
	int E_ns;                 // elements per CTA of the Navier-Stokes gradient and volume kernels
	long long elem0;          // first element (group-sorted element index)
	long long state_off;      // offset of the group's first element in state-sized arrays
	long long gmet_off;       // ... in the metric array
	long long wj_off;         // ... in the 1/(wJ) array
};

// A non-tensor-product (dense-operator) group: TET, WEDGE or PYR volumes of one p (kernels in dgpu_dense.cuh).
struct DGroup {
	int n_vs, n_vc, n_lf, n_ord;
	int n_vol, E, E_fused;      // volumes; volumes per CTA of the per-group and of the fused kernels
	long long elem0;            // first element (group-sorted index)
	long long state_off;        // in state-sized arrays
	long long gmet_off;         // per element D*D*n_vc doubles of w * metrics, component j*D+i
	const double* cv0;          // n_vc x n_vs
	const double* cv1;          // D x n_vc x n_vs
	const double* minv;         // n_vs x n_vs (M_ref^-1)
	const double* inv_J;        // per element 1 / J
	const double* minv_vol;     // per element n_vs x n_vs M^-1 when the group has a curved volume, else null
	const double* fops;         // face operator table
	const long long* fop_off;   // [(lf * n_ord + ord) * (kQMax + 1) + q_f] -> offset in fops, -1 if absent
	int vol_per_e, lift_per_e;  // shared memory per volume (doubles) of the volume and lift bodies
	int minv_identity;          // M_ref is the identity to rounding (orthonormal basis): M^-1 = 1/J
	int prism;                  // WEDGE with TRI x LINE factors: sum-factorised volume term
	int n_tvs, n_tvc, n_lvs, n_lvc;
	const double* tri0;         // n_tvc x n_tvs
	const double* tri1;         // 2 x n_tvc x n_tvs
	const double* line0;        // n_lvc x n_lvs
	const double* line1;        // n_lvc x n_lvs
	const double* ccSB0;        // n_vs x n_vs: coefficients -> Bezier coefficients (positivity), or null
	const double* ccBS0;        // n_vs x n_vs: Bezier -> coefficients
	const float* ccSB0f;        // ccSB0 in FP32 (the limiter's pre-filter)
	float pos_err;              // bound on |b_fp32 - b| / max |s| of the pre-filter's Bezier coefficients
};

struct BParams {
	double b_adv[3];
	int n_groups;             // TP groups; dense groups follow them in the tile list (group >= n_groups)
	const DGroup* dgroups;
	const BatchOps* ops;      // [group]
	const BGroup* groups;     // [group]
	const int4* elf;          // [element][kMaxLf]: (face, side, q_f, orientation)
	const long long* fbase;   // [face + 1]: first face node of the face (faces laid out by increasing q_f)
	// right-trace gather permutation per face node (side 1's trace in side 0's node order is tR[nc[fbase + i]]) and
	// its inverse (side 1's own node j holds side 0's node nc_inv[fbase + j]); both null when every face's is the
	// identity (get_operator__nc_fc_T(1, face), compute_face_rlhs_T.c:133-146)
	const int* nc = nullptr;
	const int* nc_inv = nullptr;
	const double* gmet;
	const double* inv_wJ;
	const double* fgeo;       // [node][D+1] blocks per face: (D+1) * fbase[f] + k * NF_f + i
	double* traces;           // per face: 2 NV NF_f at 2 NV fbase[f]: [side][NV][NF_f]
	double* nnf;              // per face: NV NF_f at NV fbase[f]: [NV][NF_f]
	double* vol_gl;           // state layout
	unsigned long long* max_bits;
	int* err_flag;
	unsigned long long* n_corr;
	// boundary faces (no side-1 volume), all null on a mesh without any:
	const int* fbc;           // [face]: BC code modulo BC_STEP_SC, -1 on interior faces
	const double* fext;       // per face: NV NF_f at NV fbase[f]: [NV][NF_f] exterior state at the face nodes
	BcData bc_data;
	// Navier-Stokes (BR2, dgpu_batched_ns.cuh), all null otherwise:
	double* ns_gv = nullptr;  // per element [D][NV][N] at D * its state offset: the kept volume gradient
	double* ns_gtr = nullptr; // per face: 2 D NV NF_f at 2 D NV fbase[f]: [side][D][NV][NF_f] gradient traces
	double* ns_dw = nullptr;  // per face: NV NF_f at NV fbase[f]: w_f J_f (W_R - W_L) / 2, side-0 node order
	double* ns_y = nullptr;   // per face, as ns_gtr: each side's own lifting of X at the face nodes (own node order)
	NsPhys ns = {0.0, 1.0, 1.0, kViscosityConstant, 0.0};
	double ns_eta = 0.0;      // BR2 scaling of a face's own lifting in its face gradient
	// The test case's source term (compute_source_rhs_dg_like, compute_rlhs.c:47-57) in the state layout, or null:
	// a TP element's GL nodal values of s (M^-1 tw0_vt_vc (J s) = V^-1 s: added after 1/(w J)); a dense element's
	// tw0_vt_vc (J s) = cv0^T diag(w J) s (added before M^-1).
	const double* source = nullptr;
};

// Fused tile list entry: group and first element within the group.
struct BTile {
	int group;
	int e0;
};

// ---------------------------------------------------------------------------------------------------------------
// shared-memory sizes (doubles per element) of the bodies
template <int D, int Q, int NV>
struct BSmem {
	static constexpr int N = TPShape<D, Q>::N;
	static constexpr int NFQ = TPShape<D, Q>::NF;
	static constexpr int VOL = NV * N * 2 + D * NV * N + 2 * D * NV * NFQ;   // su, st, sf, own-order traces
	static constexpr int LIFT = 3 * NV * N + 8 + 2 * D * NV * NFQ;           // sa, sb, sc, scalars, face terms
};

// ---------------------------------------------------------------------------------------------------------------
// Volume term + traces at each face's order
// ---------------------------------------------------------------------------------------------------------------
template <int D, int Q, int NV, int PDE, bool GLL_IN>
__device__ void bvol_body(const BParams& P, const BatchOps* sops, const BGroup& G, int e0, int E,
                          const double* __restrict__ u, double* base)
{
	constexpr int N = TPShape<D, Q>::N, NFQ = TPShape<D, Q>::NF;
	constexpr int PER_E = BSmem<D, Q, NV>::VOL;
	const int tid = threadIdx.x;
	const int n_here = min(E, G.n_vol - e0);
	const double* ublk = u + G.state_off + (long long)e0 * NV * N;
	for (int i = tid; i < n_here * NV * N; i += blockDim.x) {
		const int e = i / (NV * N), r = i % (NV * N);
		base[e * PER_E + r] = ublk[i];
	}
	__syncthreads();
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* su = base + e * PER_E;
	double* st = su + NV * N;
	double* sf = st + NV * N;
	double* str = sf + D * NV * N;   // [lf][NV][NFQ]
	if (GLL_IN) {
		tp_apply<D, Q, NV>(su, st, sf, sops->t.B, node, active);
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				su[k * N + node] = st[k * N + node];
		__syncthreads();
	}
	const long long v = G.elem0 + e0 + e;   // group-sorted element index
	if (active) {
		double W[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			W[k] = su[k * N + node];
		double g[D * D];
		const double* gm = P.gmet + G.gmet_off + (long long)(e0 + e) * D * D * N;
#pragma unroll
		for (int c = 0; c < D * D; ++c)
			g[c] = gm[c * N + node];
		if constexpr (PDE == kEuler) {
			double fr[D][D + 2];
			euler_flux_ref<D>(W, g, fr);
#pragma unroll
			for (int j = 0; j < D; ++j)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					sf[(j * NV + k) * N + node] = fr[j][k];
		} else {
#pragma unroll
			for (int j = 0; j < D; ++j) {
				double gb = 0.0;
#pragma unroll
				for (int i = 0; i < D; ++i)
					gb += g[j * D + i] * P.b_adv[i];
				sf[j * N + node] = gb * W[0];
			}
		}
		// traces at this element's own GL points, all faces, into shared memory
		for (int it = node; it < 2 * D * NFQ; it += N) {
			const int lf = it / NFQ, t = it % NFQ;
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
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				double s = 0.0;
#pragma unroll
				for (int m = 0; m < Q; ++m)
					s += sops->t.lb[side][m] * su[k * N + base_n + m * stride_n];
				str[(lf * NV + k) * NFQ + t] = s;
			}
		}
	}
	__syncthreads();
	if (active) {
		// volume term in GL space
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
				w[m] = sops->t.Dgl[m][a];
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				const double* f = sf + (j * NV + k) * N + b0;
#pragma unroll
				for (int m = 0; m < Q; ++m)
					acc[k] += w[m] * f[m * stride];
			}
		}
		double* vg = P.vol_gl + G.state_off + (long long)(e0 + e) * NV * N;
#pragma unroll
		for (int k = 0; k < NV; ++k)
			vg[k * N + node] = acc[k];
		// traces at each face's order: copy (q_f == Q) or tangential interpolation Q -> q_f. In 3D the
		// interpolation is separable: a thread takes one (variable, i0) column, contracts the first tangential
		// direction once per b (Q^2 FMAs) and reuses the Q partial sums for all q_f outputs i1.
		const int4* ef = P.elf + v * kMaxLf;
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int4 fd = ef[lf];
			const int qf = fd.z;
			const int nff = (D == 2 ? qf : qf * qf);
			double* dst = P.traces + 2 * NV * P.fbase[fd.x] + (long long)fd.y * NV * nff;
			const double* src = str + lf * NV * NFQ;
			if (qf == Q) {
				for (int it = node; it < NV * nff; it += N)
					dst[it] = src[it];
				continue;
			}
			const double(*I)[kQMax] = sops->Iup[qf];
			if (D == 2) {
				for (int it = node; it < NV * qf; it += N) {
					const int k = it / qf, i = it % qf;
					double s = 0.0;
#pragma unroll
					for (int a = 0; a < Q; ++a)
						s += I[i][a] * src[k * NFQ + a];
					dst[k * qf + i] = s;
				}
			} else {
				for (int it = node; it < NV * qf; it += N) {
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
	}
	__syncthreads();   // shared memory is reused by the next tile
}

// ---------------------------------------------------------------------------------------------------------------
// Face numerical flux at q_f points (faces of one q_f in [f_begin, f_end) of the face list)
// ---------------------------------------------------------------------------------------------------------------
template <int D, int NV, int PDE, int FLUX>
__device__ __forceinline__ void bface_node_rt(const BParams& P, int f, int i, int nff)
{
	const long long fb = P.fbase[f];
	const double* tL = P.traces + 2 * NV * fb;
	const double* tR = tL + NV * nff;
	double WL[NV], WR[NV], n[D];
	const double* fg = P.fgeo + (D + 1) * fb;
#pragma unroll
	for (int k = 0; k < D; ++k)
		n[k] = fg[k * nff + i];
	const int code = P.fbc ? P.fbc[f] : -1;
#pragma unroll
	for (int k = 0; k < NV; ++k)
		WL[k] = tL[k * nff + i];
	if (code < 0) {
		const int iR = P.nc ? P.nc[fb + i] : i;
#pragma unroll
		for (int k = 0; k < NV; ++k)
			WR[k] = tR[k * nff + iR];
	} else {
		// a boundary face: the boundary value of its BC from the interior trace (face_solver_T.c:203-275)
		const double* ext = P.fext + NV * fb + i;
		if constexpr (PDE == kEuler) {
			double e[NV];
#pragma unroll
			for (int k = 0; k < NV; ++k)
				e[k] = ext[k * nff];
			euler_boundary_state<D, double>(code, WL, e, n, WR, P.bc_data);
		} else {
			WR[0] = advection_boundary_value<D, double>(WL[0], ext[0], n, P.b_adv);
		}
	}
	const double sc = fg[D * nff + i];
	double* out = P.nnf + NV * fb;
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
			out[k * nff + i] = nF[k];
	} else {
		out[i] = num_flux_upwind<D>(WL[0], WR[0], n, P.b_adv) * sc;
	}
}

// ---------------------------------------------------------------------------------------------------------------
// Lift (with the transposed tangential interpolation from q_f) + M^-1 + residual | RK stage + positivity
// ---------------------------------------------------------------------------------------------------------------
template <int D, int Q, int NV, int MODE>
__device__ void blift_body(const BParams& P, const BatchOps* sops, const BGroup& G, int e0, int E, const RkArgs& rk,
                           double* base)
{
	constexpr int N = TPShape<D, Q>::N, NFQ = TPShape<D, Q>::NF;
	constexpr int PER_E = BSmem<D, Q, NV>::LIFT;
	const int tid = threadIdx.x;
	const int n_here = min(E, G.n_vol - e0);
	const int e = tid / N, node = tid % N;
	const bool active = e < n_here;
	double* sa = base + e * PER_E;
	double* sb = sa + NV * N;
	double* sc = sb + NV * N;
	int* sscale = reinterpret_cast<int*>(sc + NV * N);
	double* sg = sc + NV * N + 8;        // [lf][NV][NFQ]: E_lf^T-side face terms at this element's points
	const long long v = G.elem0 + e0 + e;
	if (active && node < 8)
		reinterpret_cast<double*>(sscale)[node] = 0.0;
	if (active) {
		// face terms at the element's own points: copy (q_f == Q) or transposed interpolation q_f -> Q
		// (separable in 3D: a thread takes one (variable, a) column, contracts i0 for every i1 once and reuses
		// the q_f partial sums for all Q outputs b).
		const int4* ef = P.elf + v * kMaxLf;
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int4 fd = ef[lf];
			const int qf = fd.z;
			const int nff = (D == 2 ? qf : qf * qf);
			const long long fb = P.fbase[fd.x];
			const double* src = P.nnf + NV * fb;
			const double sgn = (fd.y == 0 ? -1.0 : 1.0);   // side 0: rhs -= ; side 1: rhs -= (-nnf)
			// side 1 reads the face flux (side 0's node order) at its own nodes through the inverse permutation
			const int* ci = (fd.y == 1 && P.nc_inv) ? P.nc_inv + fb : nullptr;
			double* out = sg + lf * NV * NFQ;
			if (qf == Q) {
				for (int it = node; it < NV * NFQ; it += N) {
					const int k = it / NFQ, i = it % NFQ;
					out[it] = sgn * src[k * NFQ + (ci ? ci[i] : i)];
				}
				continue;
			}
			const double(*I)[kQMax] = sops->Iup[qf];
			if (D == 2) {
				for (int it = node; it < NV * Q; it += N) {
					const int k = it / Q, t = it % Q;
					double s = 0.0;
					for (int i = 0; i < qf; ++i)
						s += I[i][t] * src[k * qf + (ci ? ci[i] : i)];
					out[k * NFQ + t] = sgn * s;
				}
			} else {
				for (int it = node; it < NV * Q; it += N) {
					const int k = it / Q, a = it % Q;
					double r[kQMax];
#pragma unroll
					for (int i1 = 0; i1 < kQMax; ++i1) {
						double acc = 0.0;
						if (i1 < qf)
							for (int i0 = 0; i0 < qf; ++i0) {
								const int i = i0 + qf * i1;
								acc += I[i0][a] * src[k * nff + (ci ? ci[i] : i)];
							}
						r[i1] = acc;
					}
#pragma unroll
					for (int bb = 0; bb < Q; ++bb) {
						double s = 0.0;
#pragma unroll
						for (int i1 = 0; i1 < kQMax; ++i1)
							if (i1 < qf)
								s += I[i1][bb] * r[i1];
						out[k * NFQ + a + Q * bb] = sgn * s;
					}
				}
			}
		}
	}
	__syncthreads();

	double Rg[NV];
	if (active) {
		const double* vg = P.vol_gl + G.state_off + (long long)(e0 + e) * NV * N;
#pragma unroll
		for (int k = 0; k < NV; ++k)
			Rg[k] = vg[k * N + node];
#pragma unroll
		for (int lf = 0; lf < 2 * D; ++lf) {
			const int nd = lf >> 1;
			const int a = node_coord<Q>(node, nd);
			int t;
			if (D == 2) {
				t = (nd == 0 ? node_coord<Q>(node, 1) : node_coord<Q>(node, 0));
			} else {
				const int c0 = node_coord<Q>(node, 0), c1 = node_coord<Q>(node, 1), c2 = node_coord<Q>(node, 2);
				t = (nd == 0 ? c1 + Q * c2 : (nd == 1 ? c0 + Q * c2 : c0 + Q * c1));
			}
			const double l = sops->t.lb[lf & 1][a];
#pragma unroll
			for (int k = 0; k < NV; ++k)
				Rg[k] += l * sg[(lf * NV + k) * NFQ + t];
		}
		const double iw = P.inv_wJ[G.wj_off + (long long)(e0 + e) * N + node];
#pragma unroll
		for (int k = 0; k < NV; ++k)
			Rg[k] *= iw;
		if (P.source) {
			const double* sv = P.source + G.state_off + (long long)(e0 + e) * NV * N + node;
#pragma unroll
			for (int k = 0; k < NV; ++k)
				Rg[k] += sv[(long long)k * N];
		}
	}

	const bool need_coef = (MODE == kModeRhs) || (MODE != kModeRkGlNoMax && rk.want_max);
	unsigned long long mx = 0ull;
	double R[NV];
	if (need_coef) {
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				sa[k * N + node] = Rg[k];
		__syncthreads();
		tp_apply<D, Q, NV>(sa, sb, sc, sops->t.Binv, node, active);
		if (active) {
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				R[k] = sb[k * N + node];
				const unsigned long long bits = abs_bits(R[k]);
				mx = bits > mx ? bits : mx;
			}
		}
#pragma unroll
		for (int off = 16; off > 0; off >>= 1) {
			const unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, off);
			mx = o > mx ? o : mx;
		}
		if ((tid & 31) == 0 && mx && P.max_bits)
			atomicMax(P.max_bits, mx);
		__syncthreads();
	}
	const long long so = G.state_off + (long long)(e0 + e) * NV * N + node;
	if constexpr (MODE == kModeRhs) {
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				rk.rhs[so + (long long)k * N] = R[k];
	} else {
		double snew[NV];
		if (active) {
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				const double s = rk.u[so + (long long)k * N];
				if (rk.stage == 0) {
					rk.u0[so + (long long)k * N] = s;
					snew[k] = s + rk.dt * Rg[k];
				} else if (rk.stage == 1) {
					snew[k] = (1.0 / 4.0) * (3.0 * rk.u0[so + (long long)k * N] + s + rk.dt * Rg[k]);
				} else {
					snew[k] = (1.0 / 3.0) * (rk.u0[so + (long long)k * N] + 2.0 * s + 2.0 * rk.dt * Rg[k]);
				}
			}
		}
		if (rk.positivity) {
			if (active)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					sb[k * N + node] = snew[k];
			__syncthreads();
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
			tp_apply<D, Q, NV>(xf, tf, tmpf, sops->t.SBf, node, active);
			bool safe = true;
			if (active) {
				const float err = sops->t.pos_err;
				const float rho_lo = tf[node] - err * __int_as_float(sscale[0]);
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
					safe = 0.4f * (E_lo - ke) > 1e-5f * (fabsf(E_lo) + ke) + 1e-12f;
				}
			}
			const int unsafe = __syncthreads_or(active && !safe);
			if (unsafe) {
				int flag = 0;
				const bool corr =
					tp_positivity_exact<D, Q, NV>(sops->t.SBg, sops->t.BSg, sb, sc, sa, node, active, &flag);
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
		if (active)
#pragma unroll
			for (int k = 0; k < NV; ++k)
				rk.u[so + (long long)k * N] = snew[k];
	}
	__syncthreads();   // shared memory is reused by the next tile
}

// ---------------------------------------------------------------------------------------------------------------
// Kernels: per group, and fused persistent over all groups
// ---------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ void load_batch_ops(BatchOps* sops, const BatchOps* g)
{
	for (int i = threadIdx.x; i < (int)(sizeof(BatchOps) / 8); i += blockDim.x)
		reinterpret_cast<double*>(sops)[i] = reinterpret_cast<const double*>(g)[i];
}

template <int D, int Q, int NV, int PDE, bool GLL_IN>
__global__ void __launch_bounds__(256) bvol_group_kernel(const BParams P, int g, const double* __restrict__ u)
{
	extern __shared__ double smem[];
	BatchOps* sops = reinterpret_cast<BatchOps*>(smem);
	const BGroup G = P.groups[g];
	load_batch_ops(sops, &P.ops[g]);
	if (blockIdx.x == 0 && threadIdx.x == 0 && P.max_bits && G.elem0 == 0)   // first non-empty group
		*P.max_bits = 0ull;
	__syncthreads();
	bvol_body<D, Q, NV, PDE, GLL_IN>(P, sops, G, blockIdx.x * G.E, G.E, u, smem + sizeof(BatchOps) / 8);
}

// Minimum CTAs per SM of the per-group lift (caps its registers): 4 for the RK stages that reduce no max |rhs|
// (64 registers: twice the resident warps of the 128-register build), 2 otherwise.
template <int MODE>
struct BLiftOccupancy { static constexpr int value = (MODE == kModeRkGlNoMax) ? 4 : 2; };

template <int D, int Q, int NV, int MODE>
__global__ void __launch_bounds__(256, BLiftOccupancy<MODE>::value) blift_group_kernel(const BParams P, int g,
                                                                                      const RkArgs rk)
{
	extern __shared__ double smem[];
	BatchOps* sops = reinterpret_cast<BatchOps*>(smem);
	const BGroup G = P.groups[g];
	load_batch_ops(sops, &P.ops[g]);
	__syncthreads();
	blift_body<D, Q, NV, MODE>(P, sops, G, blockIdx.x * G.E, G.E, rk, smem + sizeof(BatchOps) / 8);
}

template <int D, int Q, int NV, bool TO_GL>
__global__ void __launch_bounds__(256) bconvert_group_kernel(const BParams P, int g, const double* __restrict__ in,
                                                               double* __restrict__ out)
{
	extern __shared__ double smem[];
	BatchOps* sops = reinterpret_cast<BatchOps*>(smem);
	double* base = smem + sizeof(BatchOps) / 8;
	const BGroup G = P.groups[g];
	load_batch_ops(sops, &P.ops[g]);
	constexpr int N = TPShape<D, Q>::N;
	constexpr int PER_E = 3 * NV * N;
	const int E = G.E, e0 = blockIdx.x * E, n_here = min(E, G.n_vol - e0);
	const double* src = in + G.state_off + (long long)e0 * NV * N;
	for (int i = threadIdx.x; i < n_here * NV * N; i += blockDim.x) {
		const int e = i / (NV * N), r = i % (NV * N);
		base[e * PER_E + r] = src[i];
	}
	__syncthreads();
	const int e = threadIdx.x / N, node = threadIdx.x % N;
	const bool active = e < n_here;
	double* sa = base + e * PER_E;
	double* sb = sa + NV * N;
	double* sc = sb + NV * N;
	tp_apply<D, Q, NV>(sa, sb, sc, TO_GL ? sops->t.B : sops->t.Binv, node, active);
	if (active)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			out[G.state_off + (long long)(e0 + e) * NV * N + (long long)k * N + node] = sb[k * N + node];
}

}  // namespace dgpu
